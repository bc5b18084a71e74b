// Device kernels of the HEOM engine: hierarchy construction, the fused
// right-hand side with its Runge-Kutta stage epilogues, the Dormand-Prince
// error norm and step control, and small helpers.
//
// Layout in HBM (the reference's `main` vector, heom_hilb.h:45-49): ADO l's
// n x n matrix is contiguous, row-major, at offset l*n^2; element e = a*n+b.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "heomgb_impl.cuh"
#include "fpconv.cuh"
#include "stage.cuh"

namespace heomgb {

LaunchCounter g_launches;


// ------------------------------------------------------------------ tensor-core commutator (tcgen05)
// For real symmetric H the commutator of ADO l needs X H for X in {R, I, R^T,
// I^T} (rho = R + iI): rows of R H and I H give -rho H, rows of R^T H = (H R)^T
// and I^T H give H rho.  One GEMM per tile: A = the 4n rows of every tile ADO
// stacked (M = 128, zero-padded), B = H (N padded to 16 or 32), K = n padded
// to 8.  Operands are split into TF32 hi + lo (3xTF32: hi*hi + hi*lo +
// lo*hi, FP32 accumulation in tensor memory), staged in shared memory in the
// K-major layout without swizzle: 8-row x 16-byte core matrices, the core
// matrices of one 8-row group adjacent along K (leading byte offset 128), row
// groups (K/4)*128 bytes apart (stride byte offset).  One thread issues the
// MMAs; completion arrives on an mbarrier; the CTA gathers the tile's bath
// terms meanwhile, then every warp reads its sub-partition of tensor-memory
// lanes back.
struct TcGeom {
  int rows_per_ado;  // 4n
  int m_total;       // rows of A: one 128-row MMA block
  int k_pad;         // n rounded up to 8
  int n_pad;         // n rounded up to 16 (16 or 32)
};
// ADOs of one tile: as many as fill one 128-row MMA (n = 8: 4, n = 12 and 16:
// 2, n = 24 and 32: 1; rows past nt * 4n are zero padding)
__host__ __device__ inline int tc_tile_ados(int n) { return 128 / (4 * n) > 0 ? 128 / (4 * n) : 1; }
__host__ __device__ inline TcGeom tc_geom(int n) {
  TcGeom t;
  t.rows_per_ado = 4 * n;
  t.m_total = 128;
  t.k_pad = (n + 7) / 8 * 8;
  t.n_pad = n <= 16 ? 16 : 32;
  return t;
}
__host__ __device__ inline size_t tc_operand_bytes(int n) {
  const TcGeom t = tc_geom(n);
  return 2 * sizeof(float) * (static_cast<size_t>(t.m_total) * t.k_pad);  // A hi + lo
}
// the four product arrays of a tile (row stride n + 1), then the partial sums
__host__ __device__ inline size_t tc_product_bytes(int n, int tile) {
  return 4 * sizeof(float) * static_cast<size_t>(tile) * n * (n + 1) + sizeof(float2) * static_cast<size_t>(tile) * n * n;
}
// x / d for 0 <= x < 2^16 and 1 <= d <= 2^12 from rd = 1.0f / d (correctly
// rounded): (x + 0.5) / d lies at least 0.5 / d away from an integer and the
// two roundings move it by less than (x / d + 1) * 2^-23, so truncation gives
// the exact quotient (checked exhaustively over that range against integer
// division)
__device__ __forceinline__ int small_div(int x, float rd) {
  return __float2int_rz(__fmul_rn(static_cast<float>(x) + 0.5f, rd));
}
__host__ __device__ inline size_t tc_b_bytes(int n) {
  const TcGeom t = tc_geom(n);
  return 2 * sizeof(float) * (static_cast<size_t>(t.n_pad) * t.k_pad);
}
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
// tcgen05 shared-memory matrix descriptor: start, leading and stride byte
// offsets in 16-byte units, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return static_cast<uint64_t>((saddr >> 4) & 0x3FFF) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFF) << 16) |
         (static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32) | (static_cast<uint64_t>(1) << 46);
}
__device__ __forceinline__ float tf32_hi(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return __uint_as_float(r);
}
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, int acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void tc_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory"); }

// Bounded wait for the completion of mbarrier phase `parity` (the MMAs of one
// tile take microseconds; the limit is orders of magnitude above that).
__device__ __forceinline__ uint32_t tc_wait(uint64_t* mbar, uint32_t parity) {
  uint32_t done = 0;
  for (int it = 0; it < (1 << 24) && !done; ++it) {
    asm volatile(
        "{\n .reg .pred q;\n mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2;\n selp.b32 %0, 1, 0, q;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(mbar)), "r"(parity));
  }
  return done;
}

// Stages A (the tile's rho rows and transposed rows, hi | lo) and, when
// build_b, B (H^T, hi | lo; it stays valid while the instance does not
// change), then thread 0 issues the MMAs and commits them to mbar.  A warp
// fills whole 8-row groups: a lane keeps its row for the group and writes
// one word of each consecutive 32-word core-matrix pair, so the stores are
// free of bank conflicts and the row arithmetic runs once per group.
__device__ __forceinline__ void tc_issue(const float2* yt, const float2* __restrict__ Hg, bool build_b, int n, int nt,
                                         float* Ah, float* Al, float* Bh, float* Bl, uint64_t* mbar, uint32_t tmem) {
  const TcGeom g = tc_geom(n);
  const int n2 = n * n, kq = g.k_pad >> 2, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  const int rr = lane >> 2, kk = lane & 3;
  const float r_n = 1.0f / n, r_rows = 1.0f / g.rows_per_ado;
  const int groups_a = g.m_total >> 3, groups = groups_a + (build_b ? g.n_pad >> 3 : 0);
  for (int grp = threadIdx.x >> 5; grp < groups; grp += nw) {
    const bool is_a = grp < groups_a;
    const int gg = is_a ? grp : grp - groups_a;
    const int m = gg * 8 + rr;
    const float2* src;
    int kstride;
    bool live, im = false;
    if (is_a) {
      const int l = small_div(m, r_rows), rem = m - l * g.rows_per_ado;
      const int part = small_div(rem, r_n), r = rem - part * n;
      live = l < nt;
      src = yt + (live ? l : 0) * n2 + (part < 2 ? r * n : r);  // row r of rho_l, or of its transpose
      kstride = part < 2 ? 1 : n;
      im = (part & 1) != 0;
    } else {
      live = m < n;
      src = Hg + (live ? m : 0);  // B[j][k] = H[k][j]
      kstride = n;
    }
    float* dh = (is_a ? Ah : Bh) + gg * kq * 32 + lane;
    float* dl = (is_a ? Al : Bl) + gg * kq * 32 + lane;
    for (int qi = 0; qi < kq; ++qi) {
      const int k = qi * 4 + kk;
      float x = 0.f;
      if (live && k < n) {
        const float2 v = is_a ? src[k * kstride] : __ldg(src + k * kstride);
        x = im ? v.y : v.x;
      }
      const float hi = tf32_hi(x);
      dh[qi * 32] = hi;
      dl[qi * 32] = x - hi;
    }
  }
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x == 0) {
    const uint32_t sbo = static_cast<uint32_t>(kq) * 128u;
    const uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(g.n_pad >> 3) << 17) |
                           (static_cast<uint32_t>(128 >> 4) << 24);
    const uint32_t ah = smem_addr(Ah), al = smem_addr(Al), bh = smem_addr(Bh), bl = smem_addr(Bl);
    for (int t = 0; t < g.m_total / 128; ++t) {
      const uint32_t d = tmem + static_cast<uint32_t>(t * g.n_pad);
      const uint32_t a_off = static_cast<uint32_t>(t) * 16u * sbo;
      for (int s = 0; s < g.k_pad / 8; ++s) {
        const uint32_t k_off = static_cast<uint32_t>(s) * 256u;
        const uint64_t dah = tc_desc(ah + a_off + k_off, 128, sbo), dal = tc_desc(al + a_off + k_off, 128, sbo);
        const uint64_t dbh = tc_desc(bh + k_off, 128, sbo), dbl = tc_desc(bl + k_off, 128, sbo);
        tc_mma(d, dah, dbh, idesc, s > 0);
        tc_mma(d, dah, dbl, idesc, 1);
        tc_mma(d, dal, dbh, idesc, 1);
      }
    }
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
        smem_addr(mbar)));
  }
}

// Waits (bounded) for the tile's MMAs and writes the products out of tensor
// memory into four FP32 arrays of nt * n * (n + 1) words (row stride n + 1):
// X1 / Y1 take the R H / I H rows (x: (I H)_rc, y: -(R H)_rc), X2 / Y2 the
// transposed H R / H I rows (x: -(H I)_cr, y: (H R)_cr); i[H, rho]_ab =
// (X1 + X2, Y1 + Y2)_ab.  The odd row stride keeps a warp's 32 rows in 32
// banks.  Returns false (CTA-uniform) if the wait gave up.
__device__ __forceinline__ bool tc_readback(int n, int nt, float* X1, float* Y1, float* X2, float* Y2,
                                            uint64_t* mbar, uint32_t tmem, uint32_t parity) {
  const TcGeom g = tc_geom(n);
  uint32_t done = 0;
  if (threadIdx.x == 0) done = tc_wait(mbar, parity);  // one waiter; the others sleep in the barrier
  done = __syncthreads_or(done);                         // its verdict for the whole CTA
  tc_fence_after();
  if (done) {
    const int warp = threadIdx.x >> 5, sp = warp & 3, lane = threadIdx.x & 31;
    const int half = warp >> 2, halves = blockDim.x >> 7;  // warps w and w + 4 share a lane sub-partition
    const int ld = n + 1, P = n * ld;
    for (int t = 0; t < g.m_total / 128; ++t) {
      const int m = t * 128 + sp * 32 + lane;
      const int l = small_div(m, 1.0f / g.rows_per_ado), rem = m - l * g.rows_per_ado;
      const int part = small_div(rem, 1.0f / n), r = rem - part * n;
      float* dst = part == 0 ? Y1 : part == 1 ? X1 : part == 2 ? Y2 : X2;
      const float sgn = (part == 0 || part == 3) ? -1.f : 1.f;
      for (int q = half; q < g.n_pad / 8; q += halves) {
        float v[8];
        tc_ld8(tmem + (static_cast<uint32_t>(sp * 32) << 16) + static_cast<uint32_t>(t * g.n_pad + 8 * q), v);
        if (l >= nt) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const int c = 8 * q + j;
          if (c < n) dst[l * P + (part < 2 ? r * ld + c : c * ld + r)] = sgn * v[j];
        }
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  return done != 0;
}

// ------------------------------------------------------------------ RHS, diagonal V
// For every bath u with diagonal V_u the coupling terms are elementwise:
// [V,X]_ab = (v_a - v_b) X_ab and {V,X}_ab = (v_a + v_b) X_ab, so element e
// only needs the neighbour ADOs of the modes whose bath couples e.
//
// Work is a list of tiles; a tile is `nt` consecutive ADOs of one instance
// (contiguous in HBM).  A CTA stages the tile's RHS input, the instance's H
// and the tile's hierarchy rows (neighbour indices, occupation numbers) in
// shared memory with coalesced loads; the commutator then reads shared memory
// only, and every bath term costs one global load of the neighbour's element.
// A single model is one instance; a batch of uneven instances (different
// n_state and depth) is many, all in the same launch.
template <typename TC, typename TB, bool HREAL>
__device__ __forceinline__ double diag_tile(const DiagInst* __restrict__ I, const DiagTile td, const Stage& st,
                                            const TB* __restrict__ y, double dt, int cur, unsigned char* smem_raw) {
  using C = cx_t<TC>;
  const int n = I->n, n2 = I->n2, K = I->K, void_idx = I->nh, tile = I->tile;
  const long long base = I->elem_off;
  const bool mt4 = (n & 3) == 0 && n >= 8;
  C* Hs = reinterpret_cast<C*>(smem_raw);        // n2
  C* yt = Hs + n2;                                // tile*n2
  C* Ds = yt + static_cast<size_t>(tile) * n2;    // tile*n2 commutators (micro-tiled path only)
  int* p1s = reinterpret_cast<int*>(Ds + (mt4 ? static_cast<size_t>(tile) * n2 : 0));  // tile*K
  int* m1s = p1s + tile * K;
  int* nks = m1s + tile * K;
  const C* __restrict__ Hg = pick<TC>(I->H, I->H_f);
  const C* __restrict__ ngd = pick<TC>(I->ngd, I->ngd_f);
  const C* __restrict__ cpl = pick<TC>(I->c_plus, I->c_plus_f);
  const C* __restrict__ cmi = pick<TC>(I->c_minus, I->c_minus_f);
  const C* __restrict__ csd = pick<TC>(I->c_sd, I->c_sd_f);
  const float2* __restrict__ term_p = I->term_p;
  const int term_first = I->term_first;
  const bool sqn = I->sqrt_norm != 0;
  const int* __restrict__ plus_ptr = I->plus_ptr;
  const int* __restrict__ plus_mode = I->plus_mode;
  const int* __restrict__ minus_ptr = I->minus_ptr;
  const int* __restrict__ minus_mode = I->minus_mode;
  const TB* __restrict__ yi = y + base;
  const int l0 = td.l0, nt = td.nt, ne = nt * n2;
  for (int i = threadIdx.x; i < n2; i += blockDim.x) Hs[i] = Hg[i];
  const TB* __restrict__ ysrc = yi + static_cast<size_t>(l0) * n2;
  for (int i = threadIdx.x; i < ne; i += blockDim.x) yt[i] = ldc<TC>(ysrc + i);
  for (int i = threadIdx.x; i < nt * K; i += blockDim.x) {
    const size_t gi = static_cast<size_t>(l0) * K + i;
    p1s[i] = __ldg(I->p1 + gi);
    m1s[i] = __ldg(I->m1 + gi);
    nks[i] = __ldg(I->nidx + gi);
  }
  __syncthreads();
  double local = 0.0;
  // Bath terms, damping and the stage epilogue of element e of tile ADO lt.
  // The neighbour loads of up to four +1 and four -1 terms are issued
  // together so their L2 latencies overlap.
  auto finish = [&](int lt, int e, int i, C D, const EpiPre& pre) {
    const C* yl = yt + lt * n2;
    // (sum_k n_k gamma_k + sum_u s_delta_u (v_a - v_b)^2) rho
    const C g0 = ngd[l0 + lt], g1 = csd[e];
    cfma(D, cx<TC>(g0.x + g1.x, g0.y + g1.y), yl[e]);
    const int* p1row = p1s + lt * K;
    const int* m1row = m1s + lt * K;
    const int* nrow = nks + lt * K;
    // an ADO without +1 neighbours (the deepest tier) skips its +1 slots
    // (they would add 0 * 0) unless the terminator stands in for them
    const bool plus_on = term_p != nullptr || __ldg(I->plus_any + l0 + lt) != 0;
    const int pb = __ldg(plus_ptr + e), pe = plus_on ? __ldg(plus_ptr + e + 1) : pb;
    const int mb = __ldg(minus_ptr + e), me = __ldg(minus_ptr + e + 1);
    for (int pp = pb, mp = mb; pp < pe || mp < me; pp += 4, mp += 4) {
      C v[8], cf[8];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int p = pp + j;
        v[j] = cx<TC>(0, 0);
        cf[j] = cx<TC>(0, 0);
        if (p < pe) {
          const int k = __ldg(plus_mode + p);
          const int lp = p1row[k];
          if (lp != void_idx) {
            v[j] = ldc<TC>(yi + static_cast<size_t>(lp) * n2 + e);
            cf[j] = cpl[p];
            if (sqn) {
              if constexpr (std::is_same<TC, double>::value) {  // sqrt(n_k + 1) c_plus from the table
                cf[j] = I->c_plus_n[static_cast<size_t>(p) * I->occ_rows + nrow[k]];
              } else {
                const TC f = sqrt(static_cast<TC>(nrow[k] + 1));
                cf[j] = cx<TC>(f * cf[j].x, f * cf[j].y);
              }
            }
          } else if (term_p) {  // truncated tier: the terminator's prediction
            const float2 t = term_p[(static_cast<size_t>(l0 + lt - term_first) * K + k) * n2 + e];
            v[j] = cx<TC>(static_cast<TC>(t.x), static_cast<TC>(t.y));
            cf[j] = cpl[p];
          }
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int p = mp + j;
        v[4 + j] = cx<TC>(0, 0);
        cf[4 + j] = cx<TC>(0, 0);
        if (p < me) {
          const int k = __ldg(minus_mode + p);
          const int lm = m1row[k];
          if (lm != void_idx) {
            v[4 + j] = ldc<TC>(yi + static_cast<size_t>(lm) * n2 + e);
            if constexpr (std::is_same<TC, double>::value) {  // n_k c_minus (or sqrt(n_k) c_minus) from the table
              cf[4 + j] = I->c_minus_n[static_cast<size_t>(p) * I->occ_rows + nrow[k]];
            } else {
              const TC nk = sqn ? sqrt(static_cast<TC>(nrow[k])) : occ<TC>(nrow[k]);
              const C cm = cmi[p];
              cf[4 + j] = cx<TC>(nk * cm.x, nk * cm.y);
            }
          }
        }
      }
      if (plus_on) {
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(D, cf[j], v[j]);
      }
#pragma unroll
      for (int j = 4; j < 8; ++j) cfma(D, cf[j], v[j]);
    }
    local += epi_post<TC>(st, static_cast<size_t>(base + static_cast<long long>(l0) * n2 + i), D, dt, cur, pre);
  };
  if (mt4) {
    // 1 x 4 register micro-tile: a thread owns 4 consecutive elements of a
    // row, so every H / rho value read from shared memory feeds 4 products.
    // The commutators go to shared memory; the bath terms and the epilogue
    // then run one element per thread, so a warp's neighbour and state
    // accesses cover consecutive elements (coalesced).
    const int ng = ne >> 2;
    for (int q = threadIdx.x; q < ng; q += blockDim.x) {
      const int i0 = q << 2;
      const int lt = i0 / n2;
      const int e0 = i0 - lt * n2;
      const int a = e0 / n, b0 = e0 - a * n;
      const C* yl = yt + lt * n2;
      C acc[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = cx<TC>(0, 0);
      if (HREAL) {
#pragma unroll 2
        for (int c = 0; c < n; ++c) {
          const TC hac = Hs[a * n + c].x;
          const C yac = yl[a * n + c];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const C ycb = yl[c * n + b0 + j];
            const TC hcb = Hs[c * n + b0 + j].x;
            acc[j].x = fma(hac, ycb.x, acc[j].x);
            acc[j].x = fma(-hcb, yac.x, acc[j].x);
            acc[j].y = fma(hac, ycb.y, acc[j].y);
            acc[j].y = fma(-hcb, yac.y, acc[j].y);
          }
        }
      } else {
        C neg[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) neg[j] = cx<TC>(0, 0);
#pragma unroll 2
        for (int c = 0; c < n; ++c) {
          const C hac = Hs[a * n + c];
          const C yac = yl[a * n + c];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            cfma(acc[j], hac, yl[c * n + b0 + j]);
            cfma(neg[j], yac, Hs[c * n + b0 + j]);
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          acc[j].x -= neg[j].x;
          acc[j].y -= neg[j].y;
        }
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) Ds[i0 + j] = cx<TC>(-acc[j].y, acc[j].x);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < ne; i += blockDim.x) {
      const int lt = i / n2;
      const EpiPre pre = epi_pre<TC>(st, static_cast<size_t>(base + static_cast<long long>(l0) * n2 + i), cur);
      finish(lt, i - lt * n2, i, Ds[i], pre);
    }
  } else {
    for (int i = threadIdx.x; i < ne; i += blockDim.x) {
      const int lt = i / n2;
      const int e = i - lt * n2;
      const int a = e / n, b = e - a * n;
      const C* yl = yt + lt * n2;
      const EpiPre pre = epi_pre<TC>(st, static_cast<size_t>(base + static_cast<long long>(l0) * n2 + i), cur);
      // i[H, rho]
      C acc = cx<TC>(0, 0);
      if (HREAL) {
#pragma unroll 4
        for (int c = 0; c < n; ++c) {
          const TC hac = Hs[a * n + c].x, hcb = Hs[c * n + b].x;
          const C ycb = yl[c * n + b], yac = yl[a * n + c];
          acc.x = fma(hac, ycb.x, acc.x);
          acc.x = fma(-hcb, yac.x, acc.x);
          acc.y = fma(hac, ycb.y, acc.y);
          acc.y = fma(-hcb, yac.y, acc.y);
        }
      } else {
        C neg = cx<TC>(0, 0);
#pragma unroll 4
        for (int c = 0; c < n; ++c) {
          cfma(acc, Hs[a * n + c], yl[c * n + b]);
          cfma(neg, yl[a * n + c], Hs[c * n + b]);
        }
        acc.x -= neg.x;
        acc.y -= neg.y;
      }
      finish(lt, e, i, cx<TC>(-acc.y, acc.x), pre);
    }
  }
  __syncthreads();
  return local;
}

template <typename TC, typename TB, int MINB>
__global__ void __launch_bounds__(256, MINB) k_rhs_diag(const DiagSet ds, const Stage st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double dt;
  int cur;
  if (!stage_prologue(st, dt, cur)) return;
  const TB* __restrict__ y = stage_input<TB>(st, cur);
  double local = 0.0;
  for (int t = blockIdx.x; t < ds.n_tiles; t += gridDim.x) {
    const DiagTile td = ds.tiles[t];
    const DiagInst* I = ds.inst + td.inst;
    if (I->h_real)
      local += diag_tile<TC, TB, true>(I, td, st, y, dt, cur, smem_raw);
    else
      local += diag_tile<TC, TB, false>(I, td, st, y, dt, cur, smem_raw);
  }
  if (st.kind == EPI_DP7) dp7_finish(st, local, ds.total);
}

// One tile of the diagonal-coupling stage with the commutators on the tensor
// cores (tc_issue / tc_readback): FP32 arithmetic (the mixed form), real
// symmetric H, a micro-tiled n_state, no terminator.  While the MMAs run, each
// thread gathers the bath terms and the damping of its elements; after the
// read-back it adds the commutator and runs the stage epilogue.  Shared memory: the tile's input
// rows, its hierarchy rows, A, B and the products.
template <typename TB>
__device__ __forceinline__ double diag_tile_tc(const DiagInst* __restrict__ I, const DiagTile td, const Stage& st,
                                               const TB* __restrict__ y, double dt, int cur, unsigned char* smem_raw,
                                               uint64_t* mbar, uint32_t tmem, uint32_t parity, bool build_b,
                                               int* fail) {
  const int n = I->n, n2 = I->n2, K = I->K, void_idx = I->nh, tile = I->tile;
  const long long base = I->elem_off;
  float2* yt = reinterpret_cast<float2*>(smem_raw);  // tile*n2
  int* p1s = reinterpret_cast<int*>(yt + static_cast<size_t>(tile) * n2);
  int* m1s = p1s + tile * K;
  int* nks = m1s + tile * K;
  unsigned char* opnd = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(nks + tile * K) + 127) & ~static_cast<uintptr_t>(127));
  float* Ah = reinterpret_cast<float*>(opnd);
  float* Al = Ah + tc_operand_bytes(n) / (2 * sizeof(float));
  float* Bh = reinterpret_cast<float*>(opnd + tc_operand_bytes(n));
  float* Bl = Bh + tc_b_bytes(n) / (2 * sizeof(float));
  const int ld = n + 1, P = n * ld;
  float* X1 = reinterpret_cast<float*>(opnd + tc_operand_bytes(n) + tc_b_bytes(n));
  float* Y1 = X1 + tile * P;
  float* X2 = Y1 + tile * P;
  float* Y2 = X2 + tile * P;
  float2* Dp = reinterpret_cast<float2*>(Y2 + tile * P);  // tile*n2 damping + bath partial sums
  const float2* __restrict__ ngd = I->ngd_f;
  const float2* __restrict__ cpl = I->c_plus_f;
  const float2* __restrict__ cmi = I->c_minus_f;
  const float2* __restrict__ csd = I->c_sd_f;
  const bool sqn = I->sqrt_norm != 0;
  const int* __restrict__ plus_ptr = I->plus_ptr;
  const int* __restrict__ plus_mode = I->plus_mode;
  const int* __restrict__ minus_ptr = I->minus_ptr;
  const int* __restrict__ minus_mode = I->minus_mode;
  const TB* __restrict__ yi = y + base;
  const int l0 = td.l0, nt = td.nt, ne = nt * n2;
  const TB* __restrict__ ysrc = yi + static_cast<size_t>(l0) * n2;
  const float r_n = 1.0f / n, r_n2 = 1.0f / n2;
  for (int i = threadIdx.x; i < ne; i += blockDim.x) yt[i] = ldc<float>(ysrc + i);
  for (int i = threadIdx.x; i < nt * K; i += blockDim.x) {
    const size_t gi = static_cast<size_t>(l0) * K + i;
    p1s[i] = __ldg(I->p1 + gi);
    m1s[i] = __ldg(I->m1 + gi);
    nks[i] = __ldg(I->nidx + gi);
  }
  __syncthreads();
  tc_issue(yt, I->H_f, build_b, n, nt, Ah, Al, Bh, Bl, mbar, tmem);
  // damping and bath terms while the tensor cores work (each thread keeps its
  // elements' partial sums in Dp and reads them back itself)
  for (int i = threadIdx.x; i < ne; i += blockDim.x) {
    float2 D = make_float2(0.f, 0.f);
    {
      const int lt = small_div(i, r_n2), e = i - lt * n2;
      const float2 g0 = ngd[l0 + lt], g1 = csd[e];
      cfma(D, make_float2(g0.x + g1.x, g0.y + g1.y), yt[i]);
      const int* p1row = p1s + lt * K;
      const int* m1row = m1s + lt * K;
      const int* nrow = nks + lt * K;
      const int pb = __ldg(plus_ptr + e), pe = __ldg(plus_ptr + e + 1);
      const int mb = __ldg(minus_ptr + e), me = __ldg(minus_ptr + e + 1);
      for (int pp = pb, mp = mb; pp < pe || mp < me; pp += 4, mp += 4) {
        float2 v[8], cf[8];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int p = pp + q;
          v[q] = cf[q] = make_float2(0.f, 0.f);
          if (p < pe) {
            const int k = __ldg(plus_mode + p);
            const int lp = p1row[k];
            if (lp != void_idx) {
              v[q] = ldc<float>(yi + static_cast<size_t>(lp) * n2 + e);
              cf[q] = cpl[p];
              if (sqn) {
                const float f = sqrtf(static_cast<float>(nrow[k] + 1));
                cf[q] = make_float2(f * cf[q].x, f * cf[q].y);
              }
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const int p = mp + q;
          v[4 + q] = cf[4 + q] = make_float2(0.f, 0.f);
          if (p < me) {
            const int k = __ldg(minus_mode + p);
            const int lm = m1row[k];
            if (lm != void_idx) {
              const float nk = sqn ? sqrtf(static_cast<float>(nrow[k])) : static_cast<float>(nrow[k]);
              const float2 cm = cmi[p];
              v[4 + q] = ldc<float>(yi + static_cast<size_t>(lm) * n2 + e);
              cf[4 + q] = make_float2(nk * cm.x, nk * cm.y);
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) cfma(D, cf[q], v[q]);
      }
    }
    Dp[i] = D;
  }
  if (!tc_readback(n, nt, X1, Y1, X2, Y2, mbar, tmem, parity)) {
    if (threadIdx.x == 0 && st.ctl) st.ctl->status = 2;  // tensor-core wait gave up
    *fail = 1;                                             // (every thread: the verdict is CTA-wide)
    return 0.0;
  }
  double local = 0.0;
  for (int i = threadIdx.x; i < ne; i += blockDim.x) {
    const int lt = small_div(i, r_n2), e = i - lt * n2, a = small_div(e, r_n);
    const int o = i + lt * n + a;  // lt * P + a * (n + 1) + b
    float2 D = Dp[i];
    D.x += X1[o] + X2[o];
    D.y += Y1[o] + Y2[o];
    const size_t gi = static_cast<size_t>(base + static_cast<long long>(l0) * n2 + i);
    const EpiPre pre = epi_pre<float>(st, gi, cur);
    local += epi_post<float>(st, gi, D, dt, cur, pre);
  }
  // no barrier here: the next tile overwrites the input rows and A only after
  // this tile's read-back barriers (their last readers ran before them), and
  // the products only after its own MMA wait
  return local;
}

// The diagonal-coupling stage with the commutators on the tensor cores
// (diag_tile_tc); every instance of the plan is eligible.  128 or 256
// threads (four warps cover the 128 tensor-memory lanes); tensor memory is
// allocated per CTA (at most 16 CTAs of 128 threads reside on an SM, each
// holding at most 32 columns: the SM's 512).  MINB 2 or 3: the register cap
// (128 or 80) the autotuner picks between.
template <typename TB, int MINB>
__global__ void __launch_bounds__(256, MINB) k_rhs_diag_tc(const DiagSet ds, const Stage st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];  // operands are rounded up to 128 bytes below
  double dt;
  int cur;
  // one verdict per CTA: another CTA of this launch may flag the controller
  // meanwhile, and the allocation below is warp-synchronous
  if (!__syncthreads_and(stage_prologue(st, dt, cur))) return;
  const TB* __restrict__ y = stage_input<TB>(st, cur);
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw + ds.smem - 16);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(smem_raw + ds.smem - 8);
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(tslot)),
                 "r"(static_cast<uint32_t>(ds.tmem_cols)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;\n");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = *tslot;
  double local = 0.0;
  uint32_t parity = 0;
  int fail = 0, b_inst = -1;
  for (int t = blockIdx.x; t < ds.n_tiles; t += gridDim.x) {
    const DiagTile td = ds.tiles[t];
    const DiagInst* I = ds.inst + td.inst;
    local += diag_tile_tc<TB>(I, td, st, y, dt, cur, smem_raw, mbar, tmem, parity, td.inst != b_inst, &fail);
    b_inst = td.inst;
    if (fail) break;
    parity ^= 1u;
  }
  // an abandoned tile's MMAs drain (bounded) before the tensor memory is freed
  if (fail) tc_wait(mbar, parity);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (threadIdx.x < 32)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem),
                 "r"(static_cast<uint32_t>(ds.tmem_cols)));
  if (st.kind == EPI_DP7) dp7_finish(st, local, ds.total);
}

// ------------------------------------------------------------------ resident Dormand-Prince interval
// The whole output interval of the mixed form's Dormand-Prince solver in one
// cooperative launch, for models small enough that the CTAs together hold
// the state in shared memory.  A CTA owns a contiguous range of ADOs and
// keeps their FP64 state and candidate state with FP32 copies, the six FP32
// stage vectors, two FP32 stage-input copies and the ADOs' bath-term table in
// shared memory; of each stage only the stage input goes through global
// memory (written for the neighbour gathers of the other CTAs and read back
// with L1-bypassing loads after a grid barrier).  The arithmetic per element
// is that of k_rhs_diag with the mixed form's Dormand-Prince epilogues
// (epi_pre/epi_post: EPI_DP, EPI_DP7), in the same operation order.  The
// error norm is summed per CTA and published; after one more barrier every
// CTA adds the partial sums in index order and runs the step controller on
// its own copy of the controller state, so all CTAs take the same decisions
// without a further exchange.  Grid barriers are bounded spins: one that runs
// out sets the failure flag and the CTAs leave.

// Per-thread element data of a resident kernel (fixed for the launch): the
// thread's elements le = threadIdx.x + r * blockDim.x, r < EPT.
template <int EPT>
struct ResElems {
  int lt[EPT], e[EPT], a[EPT], b[EPT];
  int gi[EPT];    // the element's index in the state vector
  float2 g[EPT];  // damping coefficient sum_k n_k gamma_k + the element's s_delta term
};

// The ADOs of CTA b of a resident launch: b, b + G, b + 2 G, ... (G CTAs).
// ADOs are ordered by tier and only those below the deepest have +1 terms, so
// a strided share gives every CTA the same mix of work and no CTA holds up
// the grid barriers.
struct ResAdos {
  int b0, G, na;
  __device__ __forceinline__ int ado(int lt) const { return b0 + lt * G; }
  // state index of CTA-local element le (ADO le / n2, element le % n2)
  __device__ __forceinline__ size_t gidx(int le, int n2) const {
    const int lt = le / n2;
    return static_cast<size_t>(b0 + lt * G) * n2 + (le - lt * n2);
  }
};
__device__ __forceinline__ ResAdos res_ados(int nh) {
  ResAdos A;
  A.b0 = blockIdx.x;
  A.G = gridDim.x;
  A.na = A.b0 < nh ? (nh - 1 - A.b0) / A.G + 1 : 0;
  return A;
}

// Builds the thread's element data and, for its elements, the bath-term table
// (slot-major: Toff[j * E + le] the neighbour element's offset in the state,
// -1 for none, Tcf the coefficient; slots 0-3 hold the +1 terms, 4-7 the -1
// terms, in k_rhs_diag's order; the host admits models with at most 4 + 4
// terms per element).
template <int EPT>
__device__ __forceinline__ void res_build(const DiagInst& I, const ResAdos& A, int E, int* Toff, float2* Tcf,
                                          ResElems<EPT>& el) {
  const int n = I.n, n2 = I.n2, K = I.K, void_idx = I.nh;
  const bool sqn = I.sqrt_norm != 0;
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
    const int lec = le < E ? le : 0;
    const int lt = lec / n2, e = lec - lt * n2, a = e / n;
    el.lt[r] = lt;
    el.e[r] = e;
    el.a[r] = a;
    el.b[r] = e - a * n;
    const int l = min(A.ado(lt), I.nh - 1);
    el.gi[r] = l * n2 + e;
    const float2 g0 = I.ngd_f[l], g1 = I.c_sd_f[e];
    el.g[r] = make_float2(g0.x + g1.x, g0.y + g1.y);
    if (le < E) {
      const int* __restrict__ p1row = I.p1 + static_cast<size_t>(l) * K;
      const int* __restrict__ m1row = I.m1 + static_cast<size_t>(l) * K;
      const int* __restrict__ nrow = I.nidx + static_cast<size_t>(l) * K;
      const int pb = __ldg(I.plus_ptr + e), pe = __ldg(I.plus_ptr + e + 1);
      const int mb = __ldg(I.minus_ptr + e), me = __ldg(I.minus_ptr + e + 1);
      for (int j = 0; j < 4; ++j) {
        int off = -1;
        float2 cf = make_float2(0.f, 0.f);
        const int p = pb + j;
        if (p < pe) {
          const int k = __ldg(I.plus_mode + p);
          const int lp = __ldg(p1row + k);
          if (lp != void_idx) {
            off = lp * n2 + e;
            cf = I.c_plus_f[p];
            if (sqn) {
              const float f = sqrtf(static_cast<float>(__ldg(nrow + k) + 1));
              cf = make_float2(f * cf.x, f * cf.y);
            }
          }
        }
        Toff[static_cast<size_t>(j) * E + le] = off;
        Tcf[static_cast<size_t>(j) * E + le] = cf;
      }
      for (int j = 0; j < 4; ++j) {
        int off = -1;
        float2 cf = make_float2(0.f, 0.f);
        const int p = mb + j;
        if (p < me) {
          const int k = __ldg(I.minus_mode + p);
          const int lm = __ldg(m1row + k);
          if (lm != void_idx) {
            const int nk_i = __ldg(nrow + k);
            const float nk = sqn ? sqrtf(static_cast<float>(nk_i)) : static_cast<float>(nk_i);
            const float2 cm = I.c_minus_f[p];
            off = lm * n2 + e;
            cf = make_float2(nk * cm.x, nk * cm.y);
          }
        }
        Toff[static_cast<size_t>(4 + j) * E + le] = off;
        Tcf[static_cast<size_t>(4 + j) * E + le] = cf;
      }
    }
  }
}

// Own part of a stage (commutator and damping) for the thread's elements: it
// reads only this CTA's copy Xs of the stage input (k_rhs_diag's order).
// NT > 0: the state dimension as a compile-time constant (n = NT; the loop over
// c unrolled, every index a constant offset), the same arithmetic in the same
// order as the runtime-n form.
template <bool HREAL, int EPT, int NT = 0>
__device__ __forceinline__ void res_own(const float2* Hs, const float2* Xs, int n_rt, int n2_rt, int E,
                                        const ResElems<EPT>& el, float2 (&Dp)[EPT]) {
  const int n = NT > 0 ? NT : n_rt, n2 = NT > 0 ? NT * NT : n2_rt;
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
    Dp[r] = make_float2(0.f, 0.f);
    if (le >= E) continue;
    const int lt = el.lt[r], e = el.e[r], a = el.a[r], b = el.b[r];
    const float2* yl = Xs + static_cast<size_t>(lt) * n2;
    float2 acc = make_float2(0.f, 0.f);  // [H, rho]
    if (HREAL && NT > 0) {
#pragma unroll
      for (int cc = 0; cc < (NT > 0 ? NT : 1); ++cc) {
        const float hac = Hs[a * n + cc].x, hcb = Hs[cc * n + b].x;
        const float2 ycb = yl[cc * n + b], yac = yl[a * n + cc];
        acc.x = fmaf(hac, ycb.x, acc.x);
        acc.x = fmaf(-hcb, yac.x, acc.x);
        acc.y = fmaf(hac, ycb.y, acc.y);
        acc.y = fmaf(-hcb, yac.y, acc.y);
      }
    } else if (HREAL) {
#pragma unroll 4
      for (int cc = 0; cc < n; ++cc) {
        const float hac = Hs[a * n + cc].x, hcb = Hs[cc * n + b].x;
        const float2 ycb = yl[cc * n + b], yac = yl[a * n + cc];
        acc.x = fmaf(hac, ycb.x, acc.x);
        acc.x = fmaf(-hcb, yac.x, acc.x);
        acc.y = fmaf(hac, ycb.y, acc.y);
        acc.y = fmaf(-hcb, yac.y, acc.y);
      }
    } else {
      float2 neg = make_float2(0.f, 0.f);
#pragma unroll 4
      for (int cc = 0; cc < n; ++cc) {
        cfma(acc, Hs[a * n + cc], yl[cc * n + b]);
        cfma(neg, yl[a * n + cc], Hs[cc * n + b]);
      }
      acc.x -= neg.x;
      acc.y -= neg.y;
    }
    float2 D = make_float2(-acc.y, acc.x);
    cfma(D, el.g[r], yl[e]);
    Dp[r] = D;
  }
}

// Bath terms of the thread's elements added to D: all neighbour gathers are
// issued first (L1-bypassing loads of the other CTAs' stage input Xg, which
// must not be restrict-qualified: it is written until the grid wait returns).
template <int EPT>
__device__ __forceinline__ void res_bath(const float2* Xg, const int* Toff, const float2* Tcf, int E,
                                         float2 (&D)[EPT]) {
  float2 vv[EPT][kResidentTerms];
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
#pragma unroll
    for (int j = 0; j < kResidentTerms; ++j) {
      const int off = le < E ? Toff[static_cast<size_t>(j) * E + le] : -1;
      vv[r][j] = off >= 0 ? __ldcg(Xg + off) : make_float2(0.f, 0.f);
    }
  }
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
    if (le >= E) continue;
#pragma unroll
    for (int j = 0; j < kResidentTerms; ++j) cfma(D[r], Tcf[static_cast<size_t>(j) * E + le], vv[r][j]);
  }
}

template <bool HREAL, int EPT, int NT = 0>
__global__ void __launch_bounds__(kResidentMaxBlock, 2) k_dp_resident(const ResidentArgs R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ DpCtl c;
  const DiagInst& I = R.inst;
  const int n = I.n, n2 = I.n2;
  const ResAdos A = res_ados(I.nh);  // this CTA's ADOs (strided)
  const int E = A.na * n2;
  // shared memory: H | both states (FP64) | k_1..k_6 | two stage-input copies |
  // FP32 copies of both states (Yf[i] = float(S[i]), kept with the states so
  // that no stage converts from FP64) | the bath-term table
  float2* Hs = reinterpret_cast<float2*>(smem_raw);
  double2* Sv = reinterpret_cast<double2*>(smem_raw + ((sizeof(float2) * n2 + 15) & ~static_cast<size_t>(15)));
  float2* Kv = reinterpret_cast<float2*>(Sv + 2 * static_cast<size_t>(E));
  float2* yt = Kv + 6 * static_cast<size_t>(E);
  float2* Yf = yt + 2 * static_cast<size_t>(E);
  int* Toff = reinterpret_cast<int*>(Yf + 2 * static_cast<size_t>(E));
  float2* Tcf = reinterpret_cast<float2*>(Toff + kResidentTerms * static_cast<size_t>(E));
  for (int i = threadIdx.x; i < n2; i += blockDim.x) Hs[i] = I.H_f[i];
  if (threadIdx.x == 0) c = *R.ctl;
  __syncthreads();
  {
    const int cur = c.cur;
    for (int le = threadIdx.x; le < E; le += blockDim.x) {
      const double2 v = R.S[cur][A.gidx(le, n2)];
      Sv[static_cast<size_t>(cur) * E + le] = v;
      const float2 f = to_f(v);
      Yf[static_cast<size_t>(cur) * E + le] = f;
      yt[le] = f;
    }
  }
  ResElems<EPT> el;
  res_build<EPT>(I, A, E, Toff, Tcf, el);
  unsigned long long gen = 0;
  bool ok = true;
  long long attempts = 0;
  while (!c.done) {
    if (attempts++ >= R.max_attempts) {
      __syncthreads();
      if (threadIdx.x == 0) {
        c.status = 3;
        c.done = 1;
      }
      __syncthreads();
      break;
    }
    const double dt = c.dt;
    const float fdt = static_cast<float>(dt);
    const float atol_f = static_cast<float>(c.atol), rtol_f = static_cast<float>(c.rtol);
    const int cur = c.cur;
    const double2* Sc = Sv + static_cast<size_t>(cur) * E;
    double2* Sn = Sv + static_cast<size_t>(1 - cur) * E;
    const float2* Yc = Yf + static_cast<size_t>(cur) * E;
    float2* Yn = Yf + static_cast<size_t>(1 - cur) * E;
    float local_f = 0.f;
    for (int s = 0; s < 7 && ok; ++s) {
      // stage input: own ADOs from shared memory, neighbours from global memory
      const float2* Xg = s == 0 ? R.Yb[cur] : (s < 6 ? R.Ytmp[(s - 1) & 1] : R.Yb[1 - cur]);
      const float2* Xs = yt + static_cast<size_t>(s & 1) * E;
      float2* Xn = yt + static_cast<size_t>((s + 1) & 1) * E;
      float2 D[EPT];
      res_own<HREAL, EPT, NT>(Hs, Xs, n, n2, E, el, D);
      // the other CTAs' stage input: wait for their stage s - 1 (stage 1 reads
      // the state copy, complete before the attempt)
      if (s > 0) {
        ok = grid_wait(R.bar, gen, R.spin_limit);
        if (!ok) break;
      }
      res_bath<EPT>(Xg, Toff, Tcf, E, D);
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
        if (le >= E) continue;
        // stage epilogue (epi_pre + epi_post, mixed form)
        const float2 k = make_float2(-fdt * D[r].x, -fdt * D[r].y);
        const size_t g = el.gi[r];
        if (s < 5) {  // k_s; next stage input Yb + sum_j A[s+1][j] k_j in FP32
          Kv[static_cast<size_t>(s) * E + le] = k;
          float2 y = Yc[le];
          for (int j = 0; j < s; ++j) {
            const float cj = static_cast<float>(c_dpA[s + 1][j]);
            const float2 kj = Kv[static_cast<size_t>(j) * E + le];
            y.x = fmaf(cj, kj.x, y.x);
            y.y = fmaf(cj, kj.y, y.y);
          }
          const float cs = static_cast<float>(c_dpA[s + 1][s]);
          y = make_float2(fmaf(cs, k.x, y.x), fmaf(cs, k.y, y.y));
          Xn[le] = y;
          R.Ytmp[s & 1][g] = y;
        } else if (s == 5) {  // candidate state rho + sum_j B_j k_j (float-pair sum, FP64 state)
          Kv[5 * static_cast<size_t>(E) + le] = k;
          float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
          for (int j = 0; j < 5; ++j) {
            const float2 kj = Kv[static_cast<size_t>(j) * E + le];
            ff_add_prod(hi.x, lo.x, c_dpBh[j], c_dpBl[j], kj.x);
            ff_add_prod(hi.y, lo.y, c_dpBh[j], c_dpBl[j], kj.y);
          }
          ff_add_prod(hi.x, lo.x, c_dpBh[5], c_dpBl[5], k.x);
          ff_add_prod(hi.y, lo.y, c_dpBh[5], c_dpBl[5], k.y);
          const double2 sc = Sc[le];
          const double2 hd = to_d(hi), ld = to_d(lo);
          const double2 y = make_double2((sc.x + hd.x) + ld.x, (sc.y + hd.y) + ld.y);
          Sn[le] = y;
          const float2 yb = to_f(y);
          Yn[le] = yb;
          Xn[le] = yb;
          R.Yb[1 - cur][g] = yb;
        } else {  // stage 7: e = sum_j E_j k_j in FP32, scaled squared error
          float2 ee = make_float2(0.f, 0.f);
          for (int j = 0; j < 6; ++j) {
            const float cj = static_cast<float>(c_dpE[j]);
            const float2 kj = Kv[static_cast<size_t>(j) * E + le];
            ee.x = fmaf(cj, kj.x, ee.x);
            ee.y = fmaf(cj, kj.y, ee.y);
          }
          const float c6 = static_cast<float>(c_dpE[6]);
          const float ex = fmaf(c6, k.x, ee.x), ey = fmaf(c6, k.y, ee.y);
          const float2 x1 = Xs[le];
          const float2 x2 = Yc[le];
          const float m = fmaxf(x1.x * x1.x + x1.y * x1.y, x2.x * x2.x + x2.y * x2.y);
          const float sm = atol_f + rtol_f * sqrtf(m);
          local_f += (ex * ex + ey * ey) / (sm * sm);  // the thread's terms in FP32, then FP64
        }
      }
      if (s < 6) grid_arrive(R.bar, R);
    }
    if (!ok) break;
    const double part = block_sum(f2d(local_f));
    if (threadIdx.x == 0) R.partials[blockIdx.x] = part;
    grid_arrive(R.bar, R);
    ok = grid_wait(R.bar, gen, R.spin_limit);
    if (!ok) break;
    double v = 0.0;
    for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += blockDim.x) v += __ldcg(R.partials + i);
    v = block_sum(v);
    if (threadIdx.x == 0) dp_control(&c, v, R.n_total, true);
    __syncthreads();
    // the next attempt's stage-1 input (own part): the FP32 copy of the current state
    const float2* Ynow = Yf + static_cast<size_t>(c.cur) * E;
    for (int le = threadIdx.x; le < E; le += blockDim.x) yt[le] = Ynow[le];
    __syncthreads();
  }
  if (ok) {
    const int cur = c.cur;
    for (int le = threadIdx.x; le < E; le += blockDim.x) R.S[cur][A.gidx(le, n2)] = Sv[static_cast<size_t>(cur) * E + le];
    if (blockIdx.x == 0 && threadIdx.x == 0) *R.ctl = c;
  }
}

// The fixed-step RK4 interval of the mixed form in one cooperative launch:
// n_steps steps of dt_step, then one of dt_last (fixed_step_size_solver's
// clamped last step), every stage separated by a grid barrier.  A CTA keeps
// its ADOs' FP64 state and RK4 accumulator, the state's FP32 copy, two
// stage-input copies and the bath-term table in shared memory; the stage
// inputs Y2, Y3, Y4 and the new state's FP32 copy go through global memory
// for the neighbour gathers.  Per element the arithmetic is k_rhs_diag's with
// the mixed form's RK4 epilogues (EPI_RK4_1..4), in the same order.
template <bool HREAL, int EPT, int NT = 0>
__global__ void __launch_bounds__(kResidentMaxBlock, 2) k_rk4_resident(const ResidentArgs R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DiagInst& I = R.inst;
  const int n = I.n, n2 = I.n2;
  const ResAdos A = res_ados(I.nh);  // this CTA's ADOs (strided)
  const int E = A.na * n2;
  // shared memory: H | state, accumulator (FP64) | two stage-input copies |
  // the state's FP32 copy | the bath-term table
  float2* Hs = reinterpret_cast<float2*>(smem_raw);
  double2* Sv = reinterpret_cast<double2*>(smem_raw + ((sizeof(float2) * n2 + 15) & ~static_cast<size_t>(15)));
  double2* Av = Sv + E;
  float2* yt = reinterpret_cast<float2*>(Av + E);
  float2* Yf = yt + 2 * static_cast<size_t>(E);
  int* Toff = reinterpret_cast<int*>(Yf + E);
  float2* Tcf = reinterpret_cast<float2*>(Toff + kResidentTerms * static_cast<size_t>(E));
  for (int i = threadIdx.x; i < n2; i += blockDim.x) Hs[i] = I.H_f[i];
  for (int le = threadIdx.x; le < E; le += blockDim.x) {
    const double2 v = R.S[0][A.gidx(le, n2)];
    Sv[le] = v;
    const float2 f = to_f(v);
    Yf[le] = f;
    yt[le] = f;
  }
  __syncthreads();
  ResElems<EPT> el;
  res_build<EPT>(I, A, E, Toff, Tcf, el);
  unsigned long long gen = 0;
  bool ok = true;
  for (long long step = 0; step <= R.n_steps && ok; ++step) {
    const float fdt = static_cast<float>(step < R.n_steps ? R.dt_step : R.dt_last);
    for (int s = 0; s < 4 && ok; ++s) {
      const float2* Xg = s == 0 ? R.Yb[0] : R.Ytmp[(s - 1) & 1];
      const float2* Xs = yt + static_cast<size_t>(s & 1) * E;
      float2* Xn = yt + static_cast<size_t>((s + 1) & 1) * E;
      float2 D[EPT];
      res_own<HREAL, EPT, NT>(Hs, Xs, n, n2, E, el, D);
      if (step > 0 || s > 0) {  // the other CTAs' stage input (or new state) of the last stage
        ok = grid_wait(R.bar, gen, R.spin_limit);
        if (!ok) break;
      }
      res_bath<EPT>(Xg, Toff, Tcf, E, D);
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
        if (le >= E) continue;
        const float2 k = make_float2(__fmul_rn(-fdt, D[r].x), __fmul_rn(-fdt, D[r].y));
        const size_t g = el.gi[r];
        if (s < 3) {  // rho_n = rho + c*k (FP32 from the state's copy); acc = rho + k/6 or acc += k/3
          const float cs = static_cast<float>(s == 2 ? 1.0 : 0.5);
          const float w = static_cast<float>(s == 0 ? (1.0 / 6.0) : (2.0 / 6.0));
          const float2 yf = Yf[le];
          const float2 y = make_float2(fmaf(cs, k.x, yf.x), fmaf(cs, k.y, yf.y));
          Xn[le] = y;
          R.Ytmp[s & 1][g] = y;
          double2 a = s == 0 ? Sv[le] : Av[le];
          const double2 kw = to_d(make_float2(__fmul_rn(w, k.x), __fmul_rn(w, k.y)));
          a.x += kw.x;
          a.y += kw.y;
          Av[le] = a;
        } else {  // rho = acc + k4/6
          const double2 a = Av[le];
          const double2 k6 = to_d(make_float2(__fmul_rn(1.0f / 6.0f, k.x), __fmul_rn(1.0f / 6.0f, k.y)));
          const double2 v = make_double2(a.x + k6.x, a.y + k6.y);
          Sv[le] = v;
          const float2 f = to_f(v);
          Yf[le] = f;
          Xn[le] = f;  // the next step's stage-1 input (yt[0])
          R.Yb[0][g] = f;
        }
      }
      grid_arrive(R.bar, R);
    }
  }
  if (ok)
    for (int le = threadIdx.x; le < E; le += blockDim.x) R.S[0][A.gidx(le, n2)] = Sv[le];
}

// The fixed-step RK4 interval of the FP64 form in one cooperative launch (the
// stage kernels of a small model are launch-bound): as k_rk4_resident, with
// every vector in FP64 — a CTA keeps its ADOs' state, the RK4 accumulator, two
// stage-input copies and a bath-term table with FP64 coefficients in shared
// memory; the stage inputs Y2, Y3, Y4 and the new state go through global
// memory for the neighbour gathers (the state buffer is the stage-1 input, as
// in the stage kernels).  Per element the arithmetic is k_rhs_diag's FP64
// form with the RK4 epilogues (EPI_RK4_1..4, explicit FMAs), in the same
// order, so the results are the stage kernels' bits.
template <int EPT>
__device__ __forceinline__ void res_build64(const DiagInst& I, const ResAdos& A, int E, int* Toff, double2* Tcf,
                                            ResElems<EPT>& el, double2 (&g)[EPT]) {
  const int n = I.n, n2 = I.n2, K = I.K, void_idx = I.nh;
  const bool sqn = I.sqrt_norm != 0;
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
    const int lec = le < E ? le : 0;
    const int lt = lec / n2, e = lec - lt * n2, a = e / n;
    el.lt[r] = lt;
    el.e[r] = e;
    el.a[r] = a;
    el.b[r] = e - a * n;
    const int l = min(A.ado(lt), I.nh - 1);
    el.gi[r] = l * n2 + e;
    const double2 g0 = I.ngd[l], g1 = I.c_sd[e];
    g[r] = make_double2(g0.x + g1.x, g0.y + g1.y);
    if (le < E) {
      const int* __restrict__ p1row = I.p1 + static_cast<size_t>(l) * K;
      const int* __restrict__ m1row = I.m1 + static_cast<size_t>(l) * K;
      const int* __restrict__ nrow = I.nidx + static_cast<size_t>(l) * K;
      const int pb = __ldg(I.plus_ptr + e), pe = __ldg(I.plus_ptr + e + 1);
      const int mb = __ldg(I.minus_ptr + e), me = __ldg(I.minus_ptr + e + 1);
      for (int j = 0; j < 4; ++j) {
        int off = -1;
        double2 cf = make_double2(0.0, 0.0);
        const int p = pb + j;
        if (p < pe) {
          const int k = __ldg(I.plus_mode + p);
          const int lp = __ldg(p1row + k);
          if (lp != void_idx) {
            off = lp * n2 + e;
            cf = I.c_plus[p];
            if (sqn) {
              const double f = sqrt(static_cast<double>(__ldg(nrow + k) + 1));
              cf = make_double2(f * cf.x, f * cf.y);
            }
          }
        }
        Toff[static_cast<size_t>(j) * E + le] = off;
        Tcf[static_cast<size_t>(j) * E + le] = cf;
      }
      for (int j = 0; j < 4; ++j) {
        int off = -1;
        double2 cf = make_double2(0.0, 0.0);
        const int p = mb + j;
        if (p < me) {
          const int k = __ldg(I.minus_mode + p);
          const int lm = __ldg(m1row + k);
          if (lm != void_idx) {
            const int nk_i = __ldg(nrow + k);
            const double nk = sqn ? sqrt(static_cast<double>(nk_i)) : occ<double>(nk_i);
            const double2 cm = I.c_minus[p];
            off = lm * n2 + e;
            cf = make_double2(nk * cm.x, nk * cm.y);
          }
        }
        Toff[static_cast<size_t>(4 + j) * E + le] = off;
        Tcf[static_cast<size_t>(4 + j) * E + le] = cf;
      }
    }
  }
}

template <bool HREAL, int EPT>
__global__ void __launch_bounds__(kResidentMaxBlock, 2) k_rk4_resident64(const ResidentArgs R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DiagInst& I = R.inst;
  const int n = I.n, n2 = I.n2;
  const ResAdos A = res_ados(I.nh);  // this CTA's ADOs (strided)
  const int E = A.na * n2;
  double2* S = R.S[0];  // the state: also the stage-1 input the neighbours gather
  double2* Yt[2] = {reinterpret_cast<double2*>(R.Ytmp[0]), reinterpret_cast<double2*>(R.Ytmp[1])};
  // shared memory: H | state, accumulator | two stage-input copies | the bath-term table
  double2* Hs = reinterpret_cast<double2*>(smem_raw);
  double2* Sv = Hs + n2;
  double2* Av = Sv + E;
  double2* yt = Av + E;
  double2* Tcf = yt + 2 * static_cast<size_t>(E);
  int* Toff = reinterpret_cast<int*>(Tcf + kResidentTerms * static_cast<size_t>(E));
  for (int i = threadIdx.x; i < n2; i += blockDim.x) Hs[i] = I.H[i];
  for (int le = threadIdx.x; le < E; le += blockDim.x) {
    const double2 v = S[A.gidx(le, n2)];
    Sv[le] = v;
    yt[le] = v;
  }
  __syncthreads();
  ResElems<EPT> el;
  double2 gd[EPT];
  res_build64<EPT>(I, A, E, Toff, Tcf, el, gd);
  unsigned long long gen = 0;
  bool ok = true;
  for (long long step = 0; step <= R.n_steps && ok; ++step) {
    const double dt = step < R.n_steps ? R.dt_step : R.dt_last;
    for (int s = 0; s < 4 && ok; ++s) {
      const double2* Xg = s == 0 ? S : Yt[(s - 1) & 1];
      const double2* Xs = yt + static_cast<size_t>(s & 1) * E;
      double2* Xn = yt + static_cast<size_t>((s + 1) & 1) * E;
      double2 D[EPT];
#pragma unroll
      for (int r = 0; r < EPT; ++r) {  // commutator and damping from this CTA's copy
        const int le = threadIdx.x + r * blockDim.x;
        D[r] = make_double2(0.0, 0.0);
        if (le >= E) continue;
        const int a = el.a[r], b = el.b[r];
        const double2* yl = Xs + static_cast<size_t>(el.lt[r]) * n2;
        double2 acc = make_double2(0.0, 0.0);
        if (HREAL) {
#pragma unroll 4
          for (int c = 0; c < n; ++c) {
            const double hac = Hs[a * n + c].x, hcb = Hs[c * n + b].x;
            const double2 ycb = yl[c * n + b], yac = yl[a * n + c];
            acc.x = fma(hac, ycb.x, acc.x);
            acc.x = fma(-hcb, yac.x, acc.x);
            acc.y = fma(hac, ycb.y, acc.y);
            acc.y = fma(-hcb, yac.y, acc.y);
          }
        } else {
          double2 neg = make_double2(0.0, 0.0);
#pragma unroll 4
          for (int c = 0; c < n; ++c) {
            cfma(acc, Hs[a * n + c], yl[c * n + b]);
            cfma(neg, yl[a * n + c], Hs[c * n + b]);
          }
          acc.x -= neg.x;
          acc.y -= neg.y;
        }
        double2 Dv = make_double2(-acc.y, acc.x);
        cfma(Dv, gd[r], yl[el.e[r]]);
        D[r] = Dv;
      }
      if (step > 0 || s > 0) {  // the other CTAs' stage input (or new state) of the last stage
        ok = grid_wait(R.bar, gen, R.spin_limit);
        if (!ok) break;
      }
      double2 vv[EPT][kResidentTerms];  // all gathers first (L1-bypassing: written until the wait returned)
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
#pragma unroll
        for (int j = 0; j < kResidentTerms; ++j) {
          const int off = le < E ? Toff[static_cast<size_t>(j) * E + le] : -1;
          vv[r][j] = off >= 0 ? __ldcg(Xg + off) : make_double2(0.0, 0.0);
        }
      }
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
        if (le >= E) continue;
#pragma unroll
        for (int j = 0; j < kResidentTerms; ++j) cfma(D[r], Tcf[static_cast<size_t>(j) * E + le], vv[r][j]);
        const double2 k = make_double2(-dt * D[r].x, -dt * D[r].y);
        const size_t g = el.gi[r];
        if (s < 3) {  // rho_n = rho + c*k ; acc = rho + k/6 or acc += k/3
          const double c = s == 2 ? 1.0 : 0.5;
          const double w = s == 0 ? (1.0 / 6.0) : (2.0 / 6.0);
          const double2 sv = Sv[le];
          const double2 y = make_double2(fma(c, k.x, sv.x), fma(c, k.y, sv.y));
          Xn[le] = y;
          Yt[s & 1][g] = y;
          const double2 a = s == 0 ? sv : Av[le];
          Av[le] = make_double2(fma(w, k.x, a.x), fma(w, k.y, a.y));
        } else {  // rho = acc + k4/6
          const double2 a = Av[le];
          const double2 v = make_double2(fma(1.0 / 6.0, k.x, a.x), fma(1.0 / 6.0, k.y, a.y));
          Sv[le] = v;
          Xn[le] = v;  // the next step's stage-1 input (yt[0])
          S[g] = v;
        }
      }
      grid_arrive(R.bar, R);
    }
  }
}

// The fixed-step LSRK4 interval of the mixed form in one cooperative launch
// (2N-storage RK4, lsrk4.h:32-47: buff = -buff + k or k, rho += B_s buff): a
// CTA keeps its ADOs' FP64 state (updated in place), the FP32 buffer, the
// state's FP32 copy (the stage input) and the bath-term table in shared
// memory; the new state's FP32 copy goes through global memory (alternating
// two buffers) for the neighbour gathers.  Same per-element arithmetic as
// k_rhs_diag with the mixed form's EPI_LS epilogue.
template <bool HREAL, int EPT, int NT = 0>
__global__ void __launch_bounds__(kResidentMaxBlock, 2) k_ls_resident(const ResidentArgs R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const DiagInst& I = R.inst;
  const int n = I.n, n2 = I.n2;
  const ResAdos A = res_ados(I.nh);  // this CTA's ADOs (strided)
  const int E = A.na * n2;
  // shared memory: H | state (FP64) | buffer | the state's FP32 copy | the bath-term table
  float2* Hs = reinterpret_cast<float2*>(smem_raw);
  double2* Sv = reinterpret_cast<double2*>(smem_raw + ((sizeof(float2) * n2 + 15) & ~static_cast<size_t>(15)));
  float2* Bv = reinterpret_cast<float2*>(Sv + E);
  float2* Yf = Bv + E;
  int* Toff = reinterpret_cast<int*>(Yf + E);
  float2* Tcf = reinterpret_cast<float2*>(Toff + kResidentTerms * static_cast<size_t>(E));
  for (int i = threadIdx.x; i < n2; i += blockDim.x) Hs[i] = I.H_f[i];
  for (int le = threadIdx.x; le < E; le += blockDim.x) {
    const double2 v = R.S[0][A.gidx(le, n2)];
    Sv[le] = v;
    Yf[le] = to_f(v);
  }
  __syncthreads();
  ResElems<EPT> el;
  res_build<EPT>(I, A, E, Toff, Tcf, el);
  const double B[4] = {1.0 / 3.0, 3.0 / 4.0, 2.0 / 3.0, 1.0 / 4.0};  // lsrk4.h:39-46
  unsigned long long gen = 0;
  bool ok = true;
  for (long long step = 0; step <= R.n_steps && ok; ++step) {
    const float fdt = static_cast<float>(step < R.n_steps ? R.dt_step : R.dt_last);
    for (int s = 0; s < 4 && ok; ++s) {
      const float2* Xg = R.Yb[s & 1];
      float2 D[EPT];
      // every thread's reads of Yf (its elements' rows and columns, written by
      // other threads in the epilogue below) end before that epilogue: the grid
      // wait syncs the CTA, and the first stage, which has no wait, syncs here
      res_own<HREAL, EPT, NT>(Hs, Yf, n, n2, E, el, D);
      if (step > 0 || s > 0) {
        ok = grid_wait(R.bar, gen, R.spin_limit);
        if (!ok) break;
      } else {
        __syncthreads();
      }
      res_bath<EPT>(Xg, Toff, Tcf, E, D);
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
        if (le >= E) continue;
        float2 b;
        if (s == 0) {
          b = make_float2(__fmul_rn(-fdt, D[r].x), __fmul_rn(-fdt, D[r].y));
        } else {
          const float2 pb = Bv[le];
          b = make_float2(fmaf(-fdt, D[r].x, -pb.x), fmaf(-fdt, D[r].y, -pb.y));
        }
        Bv[le] = b;
        const double2 sp = Sv[le];
        const double2 bd = to_d(b);
        const double2 v = make_double2(fma(B[s], bd.x, sp.x), fma(B[s], bd.y, sp.y));
        Sv[le] = v;
        const float2 f = to_f(v);
        Yf[le] = f;
        R.Yb[1 - (s & 1)][el.gi[r]] = f;
      }
      grid_arrive(R.bar, R);
    }
  }
  if (ok)
    for (int le = threadIdx.x; le < E; le += blockDim.x) R.S[0][A.gidx(le, n2)] = Sv[le];
}

size_t resident_smem(int n2, int ados_per_cta, int scheme) {
  const size_t E = static_cast<size_t>(ados_per_cta) * n2;
  if (scheme == kResidentRk4F64)  // H | state, accumulator, two stage inputs | table (offset, FP64 coefficient)
    return sizeof(double2) * static_cast<size_t>(n2) +
           E * (4 * sizeof(double2) + kResidentTerms * (sizeof(int) + sizeof(double2)));
  const size_t per = scheme == kResidentRk4   ? 2 * sizeof(double2) + 3 * sizeof(float2)
                     : scheme == kResidentLs  ? sizeof(double2) + 2 * sizeof(float2)
                                              : 2 * sizeof(double2) + 6 * sizeof(float2) + 4 * sizeof(float2);
  return ((sizeof(float2) * n2 + 15) & ~static_cast<size_t>(15)) +
         E * (per + kResidentTerms * (sizeof(int) + sizeof(float2)));
}

// the kernel instance for the scheme, H real or complex and EPT elements per thread
static const void* resident_kernel(int scheme, bool hreal, int ept, int n) {
  if (scheme == kResidentDpF64) return resident_dp64_kernel(hreal, ept);
  if (hreal && n == 7) {  // compile-time n for the mixed intervals of 7-level systems
    switch (scheme * 8 + ept) {
      case 1: return reinterpret_cast<const void*>(k_dp_resident<true, 1, 7>);
      case 2: return reinterpret_cast<const void*>(k_dp_resident<true, 2, 7>);
      case 9: return reinterpret_cast<const void*>(k_rk4_resident<true, 1, 7>);
      case 10: return reinterpret_cast<const void*>(k_rk4_resident<true, 2, 7>);
      case 17: return reinterpret_cast<const void*>(k_ls_resident<true, 1, 7>);
      case 18: return reinterpret_cast<const void*>(k_ls_resident<true, 2, 7>);
      default: break;
    }
  }
  switch (scheme * 8 + ept * 2 + (hreal ? 1 : 0)) {
    case 2: return reinterpret_cast<const void*>(k_dp_resident<false, 1>);
    case 3: return reinterpret_cast<const void*>(k_dp_resident<true, 1>);
    case 4: return reinterpret_cast<const void*>(k_dp_resident<false, 2>);
    case 5: return reinterpret_cast<const void*>(k_dp_resident<true, 2>);
    case 10: return reinterpret_cast<const void*>(k_rk4_resident<false, 1>);
    case 11: return reinterpret_cast<const void*>(k_rk4_resident<true, 1>);
    case 12: return reinterpret_cast<const void*>(k_rk4_resident<false, 2>);
    case 13: return reinterpret_cast<const void*>(k_rk4_resident<true, 2>);
    case 18: return reinterpret_cast<const void*>(k_ls_resident<false, 1>);
    case 19: return reinterpret_cast<const void*>(k_ls_resident<true, 1>);
    case 20: return reinterpret_cast<const void*>(k_ls_resident<false, 2>);
    case 21: return reinterpret_cast<const void*>(k_ls_resident<true, 2>);
    case 34: return reinterpret_cast<const void*>(k_rk4_resident64<false, 1>);
    case 35: return reinterpret_cast<const void*>(k_rk4_resident64<true, 1>);
    case 36: return reinterpret_cast<const void*>(k_rk4_resident64<false, 2>);
    case 37: return reinterpret_cast<const void*>(k_rk4_resident64<true, 2>);
    default: return nullptr;
  }
}

int resident_blocks_per_sm(int scheme, bool hreal, int ept, int n, int block, size_t smem) {
  const void* kern = resident_kernel(scheme, hreal, ept, n);
  if (!kern) return 0;
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block, smem) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_resident(const ResidentArgs& args, int scheme, bool hreal, int ept, int grid, int block,
                            size_t smem, cudaStream_t s) {
  const void* kern = resident_kernel(scheme, hreal, ept, args.inst.n);
  if (!kern) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  ResidentArgs a = args;
  void* params[] = {&a};
  e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(block), params, smem, s);
  ++g_launches;
  return e;
}

// ------------------------------------------------------------------ instance-resident fixed steps (batches)
// The right-hand side D of one element (e of ADO lt), k_rhs_diag's arithmetic
// in its order (commutator, damping with g = ngamma + s_delta term, summed as
// k_rhs_diag sums it, then the +1 and -1 terms in groups of four), with every
// ADO read from the bin's shared-memory copy Xi of the instance's stage input.  Slots without a term are skipped (k_rhs_diag adds
// them as 0*0, which leaves D unchanged).
// the damping coefficient of element le (e of ADO lt): the FP64 form's table entry, or the mixed
// form's FP32 sum, k_rhs_diag's operations either way
template <typename TC>
__device__ __forceinline__ cx_t<TC> local_damp(const DiagInst& I, const cx_t<TC>* Gs, int le, int lt, int e) {
  if constexpr (std::is_same<TC, double>::value) {
    return Gs[le];
  } else {
    const float2 g0 = I.ngd_f[lt], g1 = I.c_sd_f[e];
    return make_float2(g0.x + g1.x, g0.y + g1.y);
  }
}

template <typename TC>
__device__ __forceinline__ cx_t<TC> local_rhs(const DiagInst& I, const cx_t<TC>* Hi, const cx_t<TC>* Xi, int lt,
                                              int e, cx_t<TC> g) {
  using C = cx_t<TC>;
  const int n = I.n, n2 = I.n2, K = I.K, void_idx = I.nh;
  const int a = e / n, b = e - a * n;
  const C* yl = Xi + lt * n2;
  C acc = cx<TC>(0, 0);  // [H, rho]
  if (I.h_real) {
#pragma unroll 4
    for (int c = 0; c < n; ++c) {
      const TC hac = Hi[a * n + c].x, hcb = Hi[c * n + b].x;
      const C ycb = yl[c * n + b], yac = yl[a * n + c];
      acc.x = fma(hac, ycb.x, acc.x);
      acc.x = fma(-hcb, yac.x, acc.x);
      acc.y = fma(hac, ycb.y, acc.y);
      acc.y = fma(-hcb, yac.y, acc.y);
    }
  } else {
    C neg = cx<TC>(0, 0);
#pragma unroll 4
    for (int c = 0; c < n; ++c) {
      cfma(acc, Hi[a * n + c], yl[c * n + b]);
      cfma(neg, yl[a * n + c], Hi[c * n + b]);
    }
    acc.x -= neg.x;
    acc.y -= neg.y;
  }
  C D = cx<TC>(-acc.y, acc.x);
  cfma(D, g, yl[e]);  // g = ngamma of the ADO + the element's s_delta term
  const bool sqn = I.sqrt_norm != 0;
  const int* __restrict__ p1row = I.p1 + static_cast<size_t>(lt) * K;
  const int* __restrict__ m1row = I.m1 + static_cast<size_t>(lt) * K;
  const int* __restrict__ nrow = I.nidx + static_cast<size_t>(lt) * K;
  const C* __restrict__ cpl = pick<TC>(I.c_plus, I.c_plus_f);
  const C* __restrict__ cmi = pick<TC>(I.c_minus, I.c_minus_f);
  const int pb = __ldg(I.plus_ptr + e), pe = __ldg(I.plus_ptr + e + 1);
  const int mb = __ldg(I.minus_ptr + e), me = __ldg(I.minus_ptr + e + 1);
  for (int pp = pb, mp = mb; pp < pe || mp < me; pp += 4, mp += 4) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int p = pp + j;
      if (p < pe) {
        const int k = __ldg(I.plus_mode + p);
        const int lp = __ldg(p1row + k);
        if (lp != void_idx) {
          C cf = cpl[p];
          if (sqn) {
            if constexpr (std::is_same<TC, double>::value) {
              cf = I.c_plus_n[static_cast<size_t>(p) * I.occ_rows + __ldg(nrow + k)];
            } else {
              const TC f = sqrt(static_cast<TC>(__ldg(nrow + k) + 1));
              cf = cx<TC>(f * cf.x, f * cf.y);
            }
          }
          cfma(D, cf, Xi[lp * n2 + e]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int p = mp + j;
      if (p < me) {
        const int k = __ldg(I.minus_mode + p);
        const int lm = __ldg(m1row + k);
        if (lm != void_idx) {
          const int nk_i = __ldg(nrow + k);
          if constexpr (std::is_same<TC, double>::value) {
            cfma(D, I.c_minus_n[static_cast<size_t>(p) * I.occ_rows + nk_i], Xi[lm * n2 + e]);
          } else {
            const TC nk = sqn ? sqrt(static_cast<TC>(nk_i)) : occ<TC>(nk_i);
            const C cm = cmi[p];
            cfma(D, cx<TC>(nk * cm.x, nk * cm.y), Xi[lm * n2 + e]);
          }
        }
      }
    }
  }
  return D;
}

// A fixed-step interval (n_steps steps of dt_step, then one of dt_last) of
// the instances of bin blockIdx.x, RK4 or LSRK4 (SCHEME), every stage
// separated by a CTA barrier only: no instance's ADOs leave the CTA.  Shared
// memory holds H of every instance, two stage-input copies (FP64 form:
// double2; mixed form: float2) and a packed descriptor per element (instance
// slot in bits 0-7, element of the ADO in bits 8-15, ADO in bits 16-31); the
// FP64 state (updated in place), the RK4 accumulator or LSRK4 buffer and the
// state's FP32 copy (mixed form) are read and written in global memory by the
// element's owning thread only.  Per element the arithmetic is k_rhs_diag's
// with the form's RK4 (EPI_RK4_1..4) or LSRK4 (EPI_LS) epilogues, in the same
// order, so both paths give the same bits.
template <typename TC, int SCHEME>
__global__ void __launch_bounds__(512, 2) k_fixed_local(const LocalArgs A) {
  using C = cx_t<TC>;
  constexpr bool MIX = std::is_same<TC, float>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ DiagInst s_inst[kLocalMaxInst];
  __shared__ int s_ebase[kLocalMaxInst + 1], s_hbase[kLocalMaxInst + 1];
  const int i0 = A.bin_ptr[blockIdx.x];
  const int ni = min(kLocalMaxInst, A.bin_ptr[blockIdx.x + 1] - i0);
  if (static_cast<int>(threadIdx.x) < ni) s_inst[threadIdx.x] = A.inst[A.bin_inst[i0 + threadIdx.x]];
  __syncthreads();
  if (threadIdx.x == 0) {
    int e = 0, h = 0;
    for (int ii = 0; ii < ni; ++ii) {
      s_ebase[ii] = e;
      s_hbase[ii] = h;
      e += s_inst[ii].nh * s_inst[ii].n2;
      h += (s_inst[ii].n2 * static_cast<int>(sizeof(C)) + 15) / 16 * (16 / static_cast<int>(sizeof(C)));
    }
    s_ebase[ni] = e;
    s_hbase[ni] = h;
  }
  __syncthreads();
  const int E = s_ebase[ni];
  C* Hs = reinterpret_cast<C*>(smem_raw);
  C* X0 = Hs + s_hbase[ni];
  C* X1 = X0 + E;
  unsigned* desc = reinterpret_cast<unsigned*>(X1 + E);
  // FP64 form: each element's damping coefficient, summed once (two FP64 additions per element and
  // stage less on the narrow FP64 pipe); the mixed form sums it in FP32 per stage
  C* Gs = reinterpret_cast<C*>(desc + ((E + 3) & ~3));
  for (int ii = 0; ii < ni; ++ii) {
    const C* Hg = pick<TC>(s_inst[ii].H, s_inst[ii].H_f);
    for (int i = threadIdx.x; i < s_inst[ii].n2; i += blockDim.x) Hs[s_hbase[ii] + i] = Hg[i];
  }
  for (int le = threadIdx.x; le < E; le += blockDim.x) {
    int ii = 0;
    while (s_ebase[ii + 1] <= le) ++ii;
    const DiagInst& I = s_inst[ii];
    const int loc = le - s_ebase[ii];
    const int lt = loc / I.n2, e = loc - lt * I.n2;
    desc[le] = static_cast<unsigned>(ii) | (static_cast<unsigned>(e) << 8) | (static_cast<unsigned>(lt) << 16);
    if constexpr (!MIX) {
      const C g0 = I.ngd[lt], g1 = I.c_sd[e];
      Gs[le] = cx<TC>(g0.x + g1.x, g0.y + g1.y);
    }
    const size_t g = static_cast<size_t>(I.elem_off) + loc;
    if constexpr (MIX)
      X0[le] = A.Yf[g];
    else
      X0[le] = A.S[g];
  }
  __syncthreads();
  for (long long step = 0; step <= A.n_steps; ++step) {
    const double dt = step < A.n_steps ? A.dt_step : A.dt_last;
    for (int s = 0; s < 4; ++s) {
      const C* Xs = (s & 1) ? X1 : X0;
      C* Xn = (s & 1) ? X0 : X1;
      for (int le = threadIdx.x; le < E; le += blockDim.x) {
        const unsigned d = desc[le];
        const int ii = static_cast<int>(d & 0xffu), e = static_cast<int>((d >> 8) & 0xffu),
                  lt = static_cast<int>(d >> 16);
        const DiagInst& I = s_inst[ii];
        const size_t g = static_cast<size_t>(I.elem_off) + static_cast<size_t>(lt) * I.n2 + e;
        if constexpr (SCHEME == kResidentLs) {  // buff = -buff + k (or k); rho += B_s buff (lsrk4.h:32-47)
          const double Bs = s == 0 ? 1.0 / 3.0 : s == 1 ? 3.0 / 4.0 : s == 2 ? 2.0 / 3.0 : 1.0 / 4.0;
          const double2 pb = A.S[g];
          if constexpr (MIX) {  // FP32 buffer (the first half of the buffer allocation), FP64 state
            float2* buf = reinterpret_cast<float2*>(A.acc);
            const float2 pf = s == 0 ? make_float2(0.f, 0.f) : buf[g];
            const float2 D = local_rhs<TC>(I, Hs + s_hbase[ii], Xs + s_ebase[ii], lt, e, local_damp<TC>(I, Gs, le, lt, e));
            const float fdt = static_cast<float>(dt);
            const float2 b = s == 0 ? make_float2(__fmul_rn(-fdt, D.x), __fmul_rn(-fdt, D.y))
                                    : make_float2(fmaf(-fdt, D.x, -pf.x), fmaf(-fdt, D.y, -pf.y));
            buf[g] = b;
            const double2 bd = to_d(b);
            const double2 v = make_double2(fma(Bs, bd.x, pb.x), fma(Bs, bd.y, pb.y));
            A.S[g] = v;
            const float2 f = to_f(v);
            A.Yf[g] = f;
            Xn[le] = f;
          } else {
            const double2 pa = s == 0 ? make_double2(0.0, 0.0) : A.acc[g];
            const double2 D = local_rhs<TC>(I, Hs + s_hbase[ii], Xs + s_ebase[ii], lt, e, local_damp<TC>(I, Gs, le, lt, e));
            const double2 k = make_double2(-dt * D.x, -dt * D.y);
            const double2 b = s == 0 ? k : make_double2(-pa.x + k.x, -pa.y + k.y);
            A.acc[g] = b;
            const double2 v = make_double2(fma(Bs, b.x, pb.x), fma(Bs, b.y, pb.y));
            A.S[g] = v;
            Xn[le] = v;
          }
          continue;
        }
        // the epilogue's operands first, so their loads overlap the right-hand side
        const double2 pa = s == 0 ? A.S[g] : A.acc[g];
        if constexpr (MIX) {
          const float2 pf = s < 3 ? A.Yf[g] : make_float2(0.f, 0.f);
          const float2 D = local_rhs<TC>(I, Hs + s_hbase[ii], Xs + s_ebase[ii], lt, e, local_damp<TC>(I, Gs, le, lt, e));
          const float fdt = static_cast<float>(dt);
          const float2 k = make_float2(__fmul_rn(-fdt, D.x), __fmul_rn(-fdt, D.y));
          if (s < 3) {  // rho_n = rho + c*k (FP32 from the state's copy); acc = rho + k/6 or acc += k/3
            const float c = static_cast<float>(s == 2 ? 1.0 : 0.5);
            const float w = static_cast<float>(s == 0 ? (1.0 / 6.0) : (2.0 / 6.0));
            Xn[le] = make_float2(fmaf(c, k.x, pf.x), fmaf(c, k.y, pf.y));
            double2 acc = pa;
            const double2 kw = to_d(make_float2(__fmul_rn(w, k.x), __fmul_rn(w, k.y)));
            acc.x += kw.x;
            acc.y += kw.y;
            A.acc[g] = acc;
          } else {  // rho = acc + k4/6
            const double2 k6 = to_d(make_float2(__fmul_rn(1.0f / 6.0f, k.x), __fmul_rn(1.0f / 6.0f, k.y)));
            const double2 v = make_double2(pa.x + k6.x, pa.y + k6.y);
            A.S[g] = v;
            const float2 f = to_f(v);
            A.Yf[g] = f;
            Xn[le] = f;
          }
        } else {
          const double2 pb = (s == 1 || s == 2) ? A.S[g] : pa;
          const double2 D = local_rhs<TC>(I, Hs + s_hbase[ii], Xs + s_ebase[ii], lt, e, local_damp<TC>(I, Gs, le, lt, e));
          const double2 k = make_double2(-dt * D.x, -dt * D.y);
          if (s < 3) {
            const double c = s == 2 ? 1.0 : 0.5;
            const double w = s == 0 ? (1.0 / 6.0) : (2.0 / 6.0);
            Xn[le] = make_double2(fma(c, k.x, pb.x), fma(c, k.y, pb.y));
            A.acc[g] = make_double2(fma(w, k.x, pa.x), fma(w, k.y, pa.y));
          } else {
            const double2 v = make_double2(fma(1.0 / 6.0, k.x, pa.x), fma(1.0 / 6.0, k.y, pa.y));
            A.S[g] = v;
            Xn[le] = v;
          }
        }
      }
      __syncthreads();
    }
  }
}

size_t local_bin_smem(const int* n2, const int* nh, int count, bool mixed) {
  const size_t c = mixed ? sizeof(float2) : sizeof(double2);
  size_t h = 0, e = 0;
  for (int i = 0; i < count; ++i) {
    h += (static_cast<size_t>(n2[i]) * c + 15) / 16 * 16;
    e += static_cast<size_t>(n2[i]) * nh[i];
  }
  // + the FP64 form's damping table (16-byte aligned after the descriptors)
  return h + e * (2 * c + sizeof(unsigned)) + (mixed ? 0 : 12 + e * sizeof(double2));
}

static const void* local_kernel(bool mixed, int scheme) {
  if (scheme == kResidentLs)
    return mixed ? reinterpret_cast<const void*>(k_fixed_local<float, kResidentLs>)
                 : reinterpret_cast<const void*>(k_fixed_local<double, kResidentLs>);
  return mixed ? reinterpret_cast<const void*>(k_fixed_local<float, kResidentRk4>)
               : reinterpret_cast<const void*>(k_fixed_local<double, kResidentRk4>);
}

int local_blocks_per_sm(bool mixed, int scheme, int block, size_t smem) {
  const void* kern = local_kernel(mixed, scheme);
  if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)) != cudaSuccess)
    return 0;
  // every instance takes the largest shared-memory split, so that the FP64 and the mixed
  // sub-batch's bins (different sizes) can share an SM
  if (cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared) !=
      cudaSuccess)
    return 0;
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kern, block, smem) != cudaSuccess) return 0;
  return nb;
}

cudaError_t launch_local(const LocalArgs& args, bool mixed, int scheme, int grid, int block, size_t smem,
                         cudaStream_t s) {
  const void* kern = local_kernel(mixed, scheme);
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
  if (e != cudaSuccess) return e;
  LocalArgs a = args;
  void* params[] = {&a};
  e = cudaLaunchKernel(kern, dim3(grid), dim3(block), params, smem, s);
  ++g_launches;
  return e;
}

// ------------------------------------------------------------------ RHS, general V
// One CTA per ADO at a time; Phi_u / Psi_u (heom_hilb.h:311-342) and the
// commutators are formed in shared memory for any dense V_u.
template <typename TC, typename TB>
__global__ void __launch_bounds__(256) k_rhs_general(const RhsModel m, const Stage st) {
  using C = cx_t<TC>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double dt;
  int cur;
  if (!stage_prologue(st, dt, cur)) return;
  const TB* __restrict__ y = stage_input<TB>(st, cur);
  const int n = m.n, n2 = m.n2, K = m.K, void_idx = m.n_hrchy;
  C* ys = reinterpret_cast<C*>(smem_raw);
  C* Dm = ys + n2;
  C* Phi = Dm + n2;
  C* Psi = Phi + n2;
  C* T = Psi + n2;
  const C* __restrict__ H = pick<TC>(m.H, m.H_f);
  const C* __restrict__ Vall = pick<TC>(m.V, m.V_f);
  const C* __restrict__ ngd = pick<TC>(m.ngd, m.ngd_f);
  const C* __restrict__ sig = pick<TC>(m.sigma, m.sigma_f);
  const C* __restrict__ sv = pick<TC>(m.s, m.s_f);
  const C* __restrict__ av = pick<TC>(m.a, m.a_f);
  const C* __restrict__ sd = pick<TC>(m.sdelta, m.sdelta_f);
  double local = 0.0;
  for (int l = blockIdx.x; l < m.n_hrchy; l += gridDim.x) {
    const TB* yl = y + static_cast<size_t>(l) * n2;
    for (int e = threadIdx.x; e < n2; e += blockDim.x) ys[e] = ldc<TC>(yl + e);
    __syncthreads();
    const C gl = ngd[l];
    for (int e = threadIdx.x; e < n2; e += blockDim.x) {
      const int a = e / n, b = e - a * n;
      C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
      for (int c = 0; c < n; ++c) {
        cfma(acc, H[a * n + c], ys[c * n + b]);
        cfma(neg, ys[a * n + c], H[c * n + b]);
      }
      C D = cx<TC>(-(acc.y - neg.y), acc.x - neg.x);
      cfma(D, gl, ys[e]);
      Dm[e] = D;
    }
    for (int u = 0; u < m.U; ++u) {
      const C* V = Vall + static_cast<size_t>(u) * n2;
      const C sdu = sd[u];
      __syncthreads();
      if (sdu.x != TC(0) || sdu.y != TC(0)) {  // s_delta [V, [V, rho]]
        for (int e = threadIdx.x; e < n2; e += blockDim.x) {
          const int a = e / n, b = e - a * n;
          C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
          for (int c = 0; c < n; ++c) {
            cfma(acc, V[a * n + c], ys[c * n + b]);
            cfma(neg, ys[a * n + c], V[c * n + b]);
          }
          T[e] = cx<TC>(acc.x - neg.x, acc.y - neg.y);
        }
        __syncthreads();
        for (int e = threadIdx.x; e < n2; e += blockDim.x) {
          const int a = e / n, b = e - a * n;
          C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
          for (int c = 0; c < n; ++c) {
            cfma(acc, V[a * n + c], T[c * n + b]);
            cfma(neg, T[a * n + c], V[c * n + b]);
          }
          cfma(Dm[e], sdu, cx<TC>(acc.x - neg.x, acc.y - neg.y));
        }
      }
      // Phi = sum sigma_k rho_{n+1_k} + n_k s_k rho_{n-1_k};  Psi = -sum n_k a_k rho_{n-1_k}
      const int k0 = __ldg(m.bath_ptr + u), k1 = __ldg(m.bath_ptr + u + 1);
      for (int e = threadIdx.x; e < n2; e += blockDim.x) {
        C ph = cx<TC>(0, 0), ps = cx<TC>(0, 0);
        for (int k = k0; k < k1; ++k) {
          const int lp = __ldg(m.p1 + static_cast<size_t>(l) * K + k);
          if (lp != void_idx) {
            C c = sig[k];
            if (m.sqrt_norm) {
              const TC f = sqrt(static_cast<TC>(__ldg(m.nidx + static_cast<size_t>(l) * K + k) + 1));
              c = cx<TC>(f * c.x, f * c.y);
            }
            cfma(ph, c, ldc<TC>(y + static_cast<size_t>(lp) * n2 + e));
          }
        }
        for (int k = k0; k < k1; ++k) {
          const int lm = __ldg(m.m1 + static_cast<size_t>(l) * K + k);
          if (lm != void_idx) {
            const int nki = __ldg(m.nidx + static_cast<size_t>(l) * K + k);
            const TC nk = m.sqrt_norm ? sqrt(static_cast<TC>(nki)) : occ<TC>(nki);
            const C r = ldc<TC>(y + static_cast<size_t>(lm) * n2 + e);
            cfma(ph, cx<TC>(nk * sv[k].x, nk * sv[k].y), r);
            cfma(ps, cx<TC>(-nk * av[k].x, -nk * av[k].y), r);
          }
        }
        Phi[e] = ph;
        Psi[e] = ps;
      }
      __syncthreads();
      // i[V, Phi] + {V, Psi}
      for (int e = threadIdx.x; e < n2; e += blockDim.x) {
        const int a = e / n, b = e - a * n;
        C c1 = cx<TC>(0, 0), c1n = cx<TC>(0, 0), c2 = cx<TC>(0, 0);
        for (int c = 0; c < n; ++c) {
          const C vac = V[a * n + c], vcb = V[c * n + b];
          cfma(c1, vac, Phi[c * n + b]);
          cfma(c1n, Phi[a * n + c], vcb);
          cfma(c2, vac, Psi[c * n + b]);
          cfma(c2, Psi[a * n + c], vcb);
        }
        C D = Dm[e];
        D.x += -(c1.y - c1n.y) + c2.x;
        D.y += (c1.x - c1n.x) + c2.y;
        Dm[e] = D;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n2; e += blockDim.x)
      local += epilogue<TC>(st, static_cast<size_t>(l) * n2 + e, Dm[e], dt, cur);
    __syncthreads();
  }
  if (st.kind == EPI_DP7) dp7_finish(st, local, static_cast<long long>(m.n_hrchy) * n2);
}

// ------------------------------------------------------------------ RHS, Liouville (block-sparse SpMV)
// heom_liou (heom_liou.h:121-258) and heom_ado (heom_ado.h:191-202): block
// row l of the global generator is (ngamma_l I + R_0) on ADO l, sigma_k Phi_u
// on ADO n+1_k and n_k (s_k Phi_u - a_k Psi_u) on ADO n-1_k.  The blocks are
// the shared CSR superoperators scaled by per-ADO scalars, so the block
// pattern comes from the hierarchy tables and R is never materialised.
template <typename TC, typename TB>
__global__ void __launch_bounds__(256) k_rhs_liou(const RhsModel m, const Stage st) {
  using C = cx_t<TC>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double dt;
  int cur;
  if (!stage_prologue(st, dt, cur)) return;
  const TB* __restrict__ y = stage_input<TB>(st, cur);
  const int n2 = m.n2, K = m.K, void_idx = m.n_hrchy;
  C* ys = reinterpret_cast<C*>(smem_raw);
  C* Dm = ys + n2;
  C* TPhi = Dm + n2;
  C* TPsi = TPhi + n2;
  const C* __restrict__ ngd = pick<TC>(m.ngd, m.ngd_f);
  const C* __restrict__ r0v = pick<TC>(m.r0_val, m.r0_val_f);
  const C* __restrict__ phv = pick<TC>(m.phi_val, m.phi_val_f);
  const C* __restrict__ psv = pick<TC>(m.psi_val, m.psi_val_f);
  const C* __restrict__ sig = pick<TC>(m.sigma, m.sigma_f);
  const C* __restrict__ sv = pick<TC>(m.s, m.s_f);
  const C* __restrict__ av = pick<TC>(m.a, m.a_f);
  double local = 0.0;
  for (int l = blockIdx.x; l < m.n_hrchy; l += gridDim.x) {
    const TB* yl = y + static_cast<size_t>(l) * n2;
    for (int e = threadIdx.x; e < n2; e += blockDim.x) ys[e] = ldc<TC>(yl + e);
    __syncthreads();
    const C gl = ngd[l];
    for (int r = threadIdx.x; r < n2; r += blockDim.x) {
      C D = cx<TC>(0, 0);
      for (int p = __ldg(m.r0_ptr + r); p < __ldg(m.r0_ptr + r + 1); ++p) cfma(D, r0v[p], ys[__ldg(m.r0_idx + p)]);
      cfma(D, gl, ys[r]);
      Dm[r] = D;
    }
    for (int u = 0; u < m.U; ++u) {
      const int k0 = __ldg(m.bath_ptr + u), k1 = __ldg(m.bath_ptr + u + 1);
      for (int e = threadIdx.x; e < n2; e += blockDim.x) {
        C ph = cx<TC>(0, 0), ps = cx<TC>(0, 0);
        for (int k = k0; k < k1; ++k) {
          const int lp = __ldg(m.p1 + static_cast<size_t>(l) * K + k);
          if (lp != void_idx) {
            C c = sig[k];
            if (m.sqrt_norm) {
              const TC f = sqrt(static_cast<TC>(__ldg(m.nidx + static_cast<size_t>(l) * K + k) + 1));
              c = cx<TC>(f * c.x, f * c.y);
            }
            cfma(ph, c, ldc<TC>(y + static_cast<size_t>(lp) * n2 + e));
          }
        }
        for (int k = k0; k < k1; ++k) {
          const int lm = __ldg(m.m1 + static_cast<size_t>(l) * K + k);
          if (lm != void_idx) {
            const int nki = __ldg(m.nidx + static_cast<size_t>(l) * K + k);
            const TC nk = m.sqrt_norm ? sqrt(static_cast<TC>(nki)) : occ<TC>(nki);
            const C r = ldc<TC>(y + static_cast<size_t>(lm) * n2 + e);
            cfma(ph, cx<TC>(nk * sv[k].x, nk * sv[k].y), r);
            cfma(ps, cx<TC>(-nk * av[k].x, -nk * av[k].y), r);
          }
        }
        TPhi[e] = ph;
        TPsi[e] = ps;
      }
      __syncthreads();
      const int* pp = m.phi_ptr + static_cast<size_t>(u) * (n2 + 1);
      const int* qp = m.psi_ptr + static_cast<size_t>(u) * (n2 + 1);
      for (int r = threadIdx.x; r < n2; r += blockDim.x) {
        C D = Dm[r];
        for (int p = __ldg(pp + r); p < __ldg(pp + r + 1); ++p) cfma(D, phv[p], TPhi[__ldg(m.phi_idx + p)]);
        for (int p = __ldg(qp + r); p < __ldg(qp + r + 1); ++p) cfma(D, psv[p], TPsi[__ldg(m.psi_idx + p)]);
        Dm[r] = D;
      }
      __syncthreads();
    }
    for (int e = threadIdx.x; e < n2; e += blockDim.x)
      local += epilogue<TC>(st, static_cast<size_t>(l) * n2 + e, Dm[e], dt, cur);
    __syncthreads();
  }
  if (st.kind == EPI_DP7) dp7_finish(st, local, static_cast<long long>(m.n_hrchy) * n2);
}

// ------------------------------------------------------------------ RHS, Redfield
// redfield_hilb (redfield_hilb.h:66-89): one n x n state,
//   D = i[H, rho] + sum_u [V_u, Lambda_u rho - rho Lambda_u^dagger],
// with Lambda_u the Redfield operator of bath u built at set-up.  One CTA; the
// products run from shared memory; the stage epilogue is the solvers' own.
template <typename TC, typename TB>
__global__ void __launch_bounds__(256) k_rhs_redfield(const RhsModel m, const Stage st) {
  using C = cx_t<TC>;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double dt;
  int cur;
  if (!stage_prologue(st, dt, cur)) return;
  const TB* __restrict__ y = stage_input<TB>(st, cur);
  const int n = m.n, n2 = m.n2;
  C* ys = reinterpret_cast<C*>(smem_raw);
  C* Dm = ys + n2;
  C* T = Dm + n2;
  const C* __restrict__ H = pick<TC>(m.H, m.H_f);
  const C* __restrict__ Vall = pick<TC>(m.V, m.V_f);
  const C* __restrict__ Lall = pick<TC>(m.lam, m.lam_f);
  const C* __restrict__ LDall = pick<TC>(m.lamd, m.lamd_f);
  double local = 0.0;
  if (blockIdx.x == 0) {
    for (int e = threadIdx.x; e < n2; e += blockDim.x) ys[e] = ldc<TC>(y + e);
    __syncthreads();
    for (int e = threadIdx.x; e < n2; e += blockDim.x) {  // i[H, rho]
      const int a = e / n, b = e - a * n;
      C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
      for (int c = 0; c < n; ++c) {
        cfma(acc, H[a * n + c], ys[c * n + b]);
        cfma(neg, ys[a * n + c], H[c * n + b]);
      }
      Dm[e] = cx<TC>(-(acc.y - neg.y), acc.x - neg.x);
    }
    for (int u = 0; u < m.U; ++u) {
      const C* V = Vall + static_cast<size_t>(u) * n2;
      const C* L = Lall + static_cast<size_t>(u) * n2;
      const C* LD = LDall + static_cast<size_t>(u) * n2;
      __syncthreads();
      for (int e = threadIdx.x; e < n2; e += blockDim.x) {  // T = Lambda rho - rho Lambda^dagger
        const int a = e / n, b = e - a * n;
        C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
        for (int c = 0; c < n; ++c) {
          cfma(acc, L[a * n + c], ys[c * n + b]);
          cfma(neg, ys[a * n + c], LD[c * n + b]);
        }
        T[e] = cx<TC>(acc.x - neg.x, acc.y - neg.y);
      }
      __syncthreads();
      for (int e = threadIdx.x; e < n2; e += blockDim.x) {  // D += [V, T]
        const int a = e / n, b = e - a * n;
        C acc = cx<TC>(0, 0), neg = cx<TC>(0, 0);
        for (int c = 0; c < n; ++c) {
          cfma(acc, V[a * n + c], T[c * n + b]);
          cfma(neg, T[a * n + c], V[c * n + b]);
        }
        C D = Dm[e];
        D.x += acc.x - neg.x;
        D.y += acc.y - neg.y;
        Dm[e] = D;
      }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < n2; e += blockDim.x) local += epilogue<TC>(st, static_cast<size_t>(e), Dm[e], dt, cur);
  }
  if (st.kind == EPI_DP7) dp7_finish(st, local, static_cast<long long>(n2));
}

// ------------------------------------------------------------------ launch configuration
int rhs_block_size(const RhsModel& m, int path) {
  if (path != PATH_DIAG) {
    int b = 32;
    while (b < m.n2 && b < 256) b <<= 1;
    return b;
  }
  return 128;
}

int rhs_grid_size(const RhsModel& m, int path, int block, int n_sm) {
  (void)block;
  if (path == PATH_REDFIELD) return 1;
  const int per_sm = 4;
  return static_cast<int>(std::min<long long>(m.n_hrchy, static_cast<long long>(n_sm) * per_sm * 4));
}

size_t rhs_smem_bytes(const RhsModel& m, int path, bool mixed) {
  const size_t cb = mixed ? sizeof(float2) : sizeof(double2);
  if (path == PATH_GENERAL) return 5 * cb * m.n2;
  if (path == PATH_LIOU) return 4 * cb * m.n2;
  if (path == PATH_REDFIELD) return 3 * cb * m.n2;
  return 0;
}

size_t diag_tile_smem_tc(int n, int K, int tile) {
  const size_t n2 = static_cast<size_t>(n) * n;
  size_t b = sizeof(float2) * n2 * tile + 3 * sizeof(int) * static_cast<size_t>(tile) * K;
  b = (b + 127) / 128 * 128;
  b += tc_operand_bytes(n) + tc_b_bytes(n) + tc_product_bytes(n, tile);
  return (b + 15) / 16 * 16 + 128 + 16;  // alignment slack, then the mbarrier and tensor-memory address slot
}

int tc_tile(int n) { return tc_tile_ados(n); }
int tc_tmem_cols(int n) {
  const TcGeom g = tc_geom(n);
  int need = g.m_total / 128 * g.n_pad, c = 32;
  while (c < need) c <<= 1;
  return c;
}

size_t diag_tile_smem(int n2, int K, int tile, bool mixed) {
  const size_t cb = mixed ? sizeof(float2) : sizeof(double2);
  const int n = static_cast<int>(std::lround(std::sqrt(static_cast<double>(n2))));
  const bool mt4 = (n & 3) == 0 && n >= 8;  // diag_tile's micro-tiled path stages its commutators
  return cb * static_cast<size_t>(n2) * (1 + tile * (mt4 ? 2 : 1)) + 3 * sizeof(int) * static_cast<size_t>(tile) * K;
}

template <typename TC, typename TB>
static cudaError_t launch_typed(const RhsModel& m, const DiagSet* ds, const Stage& st, int path, int grid, int block,
                                cudaStream_t s) {
  const size_t smem = rhs_smem_bytes(m, path, std::is_same<TC, float>::value);
  if (path == PATH_DIAG) {
    if constexpr (std::is_same<TC, float>::value && std::is_same<TB, float2>::value)
      if (ds->sites) return launch_sites(*ds, st, grid, block, s);  // counts its own launch
    const size_t dsm = ds->smem;
    // the register-capped variant exists for the FP32 arithmetic only (the
    // FP64 kernel would spill at 80 registers)
    auto kern = k_rhs_diag<TC, TB, 1>;
    if constexpr (std::is_same<TC, float>::value) {
      if (ds->min_blocks == 3) kern = k_rhs_diag<TC, TB, 3>;
      if (ds->min_blocks == 4) kern = k_rhs_diag<TC, TB, 4>;  // 64 registers: 32 warps per SM
      if (ds->tcore) kern = ds->min_blocks == 3 ? k_rhs_diag_tc<TB, 3> : k_rhs_diag_tc<TB, 2>;
    }
    if (dsm > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(dsm));
      if (e != cudaSuccess) return e;
    }
    kern<<<grid, block, dsm, s>>>(*ds, st);
  } else if (path == PATH_GENERAL) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_rhs_general<TC, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
      if (e != cudaSuccess) return e;
    }
    k_rhs_general<TC, TB><<<grid, block, smem, s>>>(m, st);
  } else if (path == PATH_REDFIELD) {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_rhs_redfield<TC, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
      if (e != cudaSuccess) return e;
    }
    k_rhs_redfield<TC, TB><<<1, block, smem, s>>>(m, st);
  } else {
    if (smem > 48 * 1024) {
      cudaError_t e = cudaFuncSetAttribute(k_rhs_liou<TC, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           static_cast<int>(smem));
      if (e != cudaSuccess) return e;
    }
    k_rhs_liou<TC, TB><<<grid, block, smem, s>>>(m, st);
  }
  ++g_launches;
  return cudaGetLastError();
}

cudaError_t launch_rhs(const RhsModel& m, const DiagSet* ds, const Stage& st, int path, bool mixed, bool in_double,
                       int grid, int block, cudaStream_t s) {
  if (path == PATH_DIAG && !ds) return cudaErrorInvalidValue;
  if (!mixed) return launch_typed<double, double2>(m, ds, st, path, grid, block, s);
  if (in_double) return launch_typed<float, double2>(m, ds, st, path, grid, block, s);
  return launch_typed<float, float2>(m, ds, st, path, grid, block, s);
}

// ------------------------------------------------------------------ hierarchy on the device
// Order of the reference's breadth-first enumeration (hrchy_space.cc:160-198):
// tier |n| ascending, and within a tier descending lexicographic order of n.
// binom is a (dim x dim) table of C(a, b), saturated where it would overflow.
__device__ __forceinline__ long long binom_at(const long long* t, int dim, int a, int b) {
  if (a < 0 || b < 0 || b > a) return 0;
  return t[static_cast<size_t>(a) * dim + b];
}

// Rank of multi-index row (with `delta` added at mode `kk`) of total `tier`.
__device__ int rank_of(const int* row, int K, int kk, int delta, int tier, const long long* bt, int bd) {
  long long r = tier > 0 ? binom_at(bt, bd, K + tier - 1, K) : 0;
  int s = tier;
  for (int i = 0; i < K - 1; ++i) {
    const int mi = row[i] + (i == kk ? delta : 0);
    const int p = K - i - 1;
    const int x = s - mi - 1;
    if (x >= 0) r += binom_at(bt, bd, x + p, p);
    s -= mi;
    if (s == 0) break;
  }
  return static_cast<int>(r);
}

__global__ void k_hrchy_unrank(int K, int n_hrchy, const long long* bt, int bd, int* nidx) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n_hrchy) return;
  int* row = nidx + static_cast<size_t>(l) * K;
  int d = 0;
  while (binom_at(bt, bd, K + d, K) <= l) ++d;
  long long r = l - (d > 0 ? binom_at(bt, bd, K + d - 1, K) : 0);
  int s = d;
  for (int i = 0; i < K; ++i) {
    const int p = K - i - 1;
    if (p == 0) {
      row[i] = s;
      break;
    }
    int v = s;
    for (; v > 0; --v) {
      const long long cnt = binom_at(bt, bd, s - v + p - 1, p - 1);
      if (r < cnt) break;
      r -= cnt;
    }
    row[i] = v;
    s -= v;
  }
}

__global__ void k_hrchy_links(int K, int depth, int n_hrchy, const long long* bt, int bd, const int* nidx, int* p1,
                              int* m1) {
  const long long gid = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x;
  const long long total = static_cast<long long>(n_hrchy + 1) * K;
  if (gid >= total) return;
  const int l = static_cast<int>(gid / K), k = static_cast<int>(gid - static_cast<long long>(l) * K);
  if (l == n_hrchy) {  // sentinel row
    p1[gid] = n_hrchy;
    m1[gid] = n_hrchy;
    return;
  }
  const int* row = nidx + static_cast<size_t>(l) * K;
  int tier = 0;
  for (int i = 0; i < K; ++i) tier += row[i];
  p1[gid] = (tier + 1 <= depth) ? rank_of(row, K, k, +1, tier + 1, bt, bd) : n_hrchy;
  m1[gid] = (row[k] > 0) ? rank_of(row, K, k, -1, tier - 1, bt, bd) : n_hrchy;
}

cudaError_t launch_hrchy_build(int K, int depth, int n_hrchy, const long long* binom, int binom_dim, int* nidx,
                               int* p1, int* m1, cudaStream_t s) {
  if (K > 0) {
    k_hrchy_unrank<<<(n_hrchy + 127) / 128, 128, 0, s>>>(K, n_hrchy, binom, binom_dim, nidx);
    ++g_launches;
    const long long total = static_cast<long long>(n_hrchy + 1) * K;
    k_hrchy_links<<<static_cast<unsigned>((total + 255) / 256), 256, 0, s>>>(K, depth, n_hrchy, binom, binom_dim,
                                                                            nidx, p1, m1);
    ++g_launches;
  }
  return cudaGetLastError();
}

// ngamma_diag[l] = sum_k n_k gamma_kk, mode by mode without contraction (heom.h:94-104).
__global__ void k_ngd(int K, int n_hrchy, const int* nidx, const double2* gdiag, double2* ngd, float2* ngd_f) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n_hrchy) return;
  double re = 0.0, im = 0.0;
  for (int k = 0; k < K; ++k) {
    const double nk = static_cast<double>(nidx[static_cast<size_t>(l) * K + k]);
    re = __dadd_rn(re, __dmul_rn(nk, gdiag[k].x));
    im = __dadd_rn(im, __dmul_rn(nk, gdiag[k].y));
  }
  ngd[l] = make_double2(re, im);
  ngd_f[l] = make_float2(static_cast<float>(re), static_cast<float>(im));
}

cudaError_t launch_ngd(int K, int n_hrchy, const int* nidx, const double2* gdiag, double2* ngd, float2* ngd_f,
                       cudaStream_t s) {
  k_ngd<<<(n_hrchy + 127) / 128, 128, 0, s>>>(K, n_hrchy, nidx, gdiag, ngd, ngd_f);
  ++g_launches;
  return cudaGetLastError();
}

// plus_any[l] = 1 if ADO l has any +1 neighbour (ptr_p1 not the sentinel)
__global__ void k_plus_any(int K, int n_hrchy, const int* p1, int* out) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= n_hrchy) return;
  int any = 0;
  for (int k = 0; k < K; ++k) any |= p1[static_cast<size_t>(l) * K + k] != n_hrchy;
  out[l] = any;
}

// The FP64 coefficient tables of DiagInst::c_minus_n / c_plus_n, with the
// same operations the stage kernels apply per term (so the products agree bit
// for bit): n_k * c, sqrt(n_k) * c or sqrt(n_k + 1) * c.
__global__ void k_scaled_coef(int n_terms, int rows, const double2* c, double2* out, int plus, int sqn) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_terms * rows) return;
  const int p = i / rows, nk = i - p * rows;
  const double2 cm = c[p];
  const double f = plus ? sqrt(static_cast<double>(nk + 1)) : (sqn ? sqrt(static_cast<double>(nk)) : occ<double>(nk));
  out[i] = make_double2(f * cm.x, f * cm.y);
}

cudaError_t launch_scaled_coef(int n_terms, int rows, const double2* c, double2* out, bool plus, bool sqn,
                               cudaStream_t s) {
  const int total = n_terms * rows;
  if (total <= 0) return cudaSuccess;
  k_scaled_coef<<<(total + 127) / 128, 128, 0, s>>>(n_terms, rows, c, out, plus ? 1 : 0, sqn ? 1 : 0);
  ++g_launches;
  return cudaGetLastError();
}

cudaError_t launch_plus_any(int K, int n_hrchy, const int* p1, int* out, cudaStream_t s) {
  if (n_hrchy <= 0) return cudaSuccess;
  k_plus_any<<<(n_hrchy + 127) / 128, 128, 0, s>>>(K, n_hrchy, p1, out);
  ++g_launches;
  return cudaGetLastError();
}

__global__ void k_to_bulk(const double2* src, float2* dst, long long n) {
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 v = src[i];
    dst[i] = to_f(v);
  }
}

cudaError_t launch_to_bulk(const double2* src, float2* dst, long long n, cudaStream_t s) {
  const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 8)));
  k_to_bulk<<<grid, 256, 0, s>>>(src, dst, n);
  ++g_launches;
  return cudaGetLastError();
}

// out_l = in_l^T for `count` consecutive n x n blocks: the reference's
// col_major storage of the ADOs <-> the row-major layout the kernels use.
// Out of place; one thread per element, reads coalesced.
__global__ void k_transpose_ados(const double2* __restrict__ in, double2* __restrict__ out, int n, long long count) {
  const long long n2 = static_cast<long long>(n) * n, total = n2 * count;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < total;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const long long l = i / n2;
    const int e = static_cast<int>(i - l * n2);
    const int a = e / n, b = e - a * n;
    out[l * n2 + static_cast<long long>(b) * n + a] = in[i];
  }
}

cudaError_t launch_transpose_ados(const double2* in, double2* out, int n, long long count, cudaStream_t s) {
  const long long total = static_cast<long long>(n) * n * count;
  if (total <= 0) return cudaSuccess;
  const int grid = static_cast<int>(std::max<long long>(1, std::min<long long>((total + 255) / 256, 152 * 8)));
  k_transpose_ados<<<grid, 256, 0, s>>>(in, out, n, count);
  ++g_launches;
  return cudaGetLastError();
}

// ------------------------------------------------------------------ arithmetic peak probe
// Register-only FMA chains (8 independent per thread, one store per thread):
// the FP64 and FP32 FMA rates of this GPU, the denominators of the
// compute-bound roofline of the plain FP64 form.
template <typename T>
__global__ void k_fma_chain(T* out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b);
    x1 = fma(x1, a, b);
    x2 = fma(x2, a, b);
    x3 = fma(x3, a, b);
    x4 = fma(x4, a, b);
    x5 = fma(x5, a, b);
    x6 = fma(x6, a, b);
    x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <typename T>
static cudaError_t time_fma(int n_sm, double* tflops, cudaStream_t s) {
  const int grid = n_sm * 8, block = 256, iters = 2048, reps = 3;
  T* d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(T) * grid * block);
  if (e != cudaSuccess) return e;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_chain<T><<<grid, block, 0, s>>>(d, iters, static_cast<T>(0.999), static_cast<T>(0.001));
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps; ++r)
    k_fma_chain<T><<<grid, block, 0, s>>>(d, iters, static_cast<T>(0.999), static_cast<T>(0.001));
  cudaEventRecord(e1, s);
  e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  g_launches += reps + 1;
  *tflops = static_cast<double>(reps) * grid * block * iters * 8.0 * 2.0 / (ms * 1e-3) / 1e12;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t probe_fma_peaks(int n_sm, double* fp64_tflops, double* fp32_tflops, cudaStream_t s) {
  cudaError_t e = time_fma<double>(n_sm, fp64_tflops, s);
  if (e != cudaSuccess) return e;
  return time_fma<float>(n_sm, fp32_tflops, s);
}

// ------------------------------------------------------------------ controller set-up
// Written by a kernel (stream-ordered, capturable) rather than by a host copy.
__global__ void k_ctl_init(DpCtl* c, double t, double dt, double t_bound, double atol, double rtol, int cur) {
  c->t = t;
  c->dt = dt;
  c->t_bound = t_bound;
  c->atol = atol;
  c->rtol = rtol;
  c->err = 0.0;
  c->dt_fixed = dt;
  c->cur = cur;
  c->count = 0;
  c->done = 0;
  c->status = 0;
  c->attempts = 0;
  c->accepted = 0;
  c->arrive = 0;
}

__global__ void k_ctl_set_fixed(DpCtl* c, double dt) { c->dt_fixed = dt; }

cudaError_t launch_ctl_init(DpCtl* c, double t, double dt, double t_bound, double atol, double rtol, int cur,
                            cudaStream_t s) {
  k_ctl_init<<<1, 1, 0, s>>>(c, t, dt, t_bound, atol, rtol, cur);
  ++g_launches;
  return cudaGetLastError();
}

cudaError_t launch_ctl_set_fixed(DpCtl* c, double dt, cudaStream_t s) {
  k_ctl_set_fixed<<<1, 1, 0, s>>>(c, dt);
  ++g_launches;
  return cudaGetLastError();
}

// ------------------------------------------------------------------ standalone error norm
// errnrm1 of linalg_engine_cuda.cu:102-201 in one launch: per-CTA partials,
// last CTA adds them in order and writes sqrt(sum/n).
__global__ void k_errnrm1(const double2* e, const double2* x1, const double2* x2, double atol, double rtol,
                          long long n, double* partials, double* out, unsigned int* counter) {
  double local = 0.0;
  for (long long i = blockIdx.x * static_cast<long long>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<long long>(gridDim.x) * blockDim.x) {
    const double2 a = e[i], b = x1[i], c = x2[i];
    const double q = hypot(a.x, a.y) / (atol + rtol * fmax(hypot(b.x, b.y), hypot(c.x, c.y)));
    local += q * q;
  }
  const double part = block_sum(local);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = part;
    __threadfence();
    last = (atomicAdd(counter, 1u) == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += blockDim.x) v += __ldcg(partials + i);
  v = block_sum(v);
  if (threadIdx.x == 0) {
    *out = sqrt(v / static_cast<double>(n));
    *counter = 0;
  }
}

int errnrm1_grid(long long n) {
  return static_cast<int>(std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 4)));
}

cudaError_t launch_errnrm1(const double2* e, const double2* x1, const double2* x2, double atol, double rtol,
                           long long n, double* partials, double* out, unsigned int* counter, int grid,
                           cudaStream_t s) {
  k_errnrm1<<<grid, 256, 0, s>>>(e, x1, x2, atol, rtol, n, partials, out, counter);
  ++g_launches;
  return cudaGetLastError();
}

}  // namespace heomgb
