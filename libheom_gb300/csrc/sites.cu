// Stage kernel for site-local baths: every bath couples through a diagonal V_u
// with a single nonzero entry (the exciton aggregates, V_j = |j><j|), the
// state's n_state a multiple of 4 (n >= 8), mixed form (FP32 stage input,
// FP64 state).  Same operator and stage epilogues as k_rhs_diag
// (heom_hilb.h:96-215 with the fused rk4 / lsrk4 / rkdp stages), with the
// work arranged for this structure:
//
// * Element (a, b) couples only to the modes of the baths at sites a and b.
//   An ADO on tier t has at most t occupied modes, so its -1 terms are read
//   from a per-ADO list of occupied modes built at set-up ({k, ptr_m1, n_k,
//   site}); an element tests each entry's site against a and b and gathers
//   only the neighbours it couples to.  ADOs with +1 neighbours (all but the
//   deepest tier) take their +1 terms from the per-element lists.
// * A thread owns a 4 x 4 block of one ADO: the commutator -i[H, rho]
//   accumulates in 16 complex registers with paired FP32 FMAs (__ffma2_rn:
//   both components of a complex value in one instruction) from H and the
//   tile's stage input in shared memory (per c: one row of H^T, one of -H,
//   four elements of row c and four of column c), and the thread then adds
//   the damping and bath terms and runs the stage epilogue row by row for the
//   same 16 elements: no shared-memory round trip for the commutators.
// * The stage epilogue is a template argument (one instance per epilogue
//   kind), so no kind switch runs per element.
// * Tiles of consecutive ADOs are staged with cp.async (16-byte copies) into
//   two alternating shared-memory buffers: the next tile's stage input and
//   records are in flight while the current tile computes, and the state
//   vectors its stage epilogue will read are prefetched into L2 with one bulk
//   prefetch per vector (cp.async.bulk.prefetch.L2).
//
// Every element's arithmetic and its order are k_rhs_diag's (commutator over
// c, then the damping, the +1 terms in list order, the -1 terms in increasing
// k; terms with no neighbour are skipped, which the other kernels add as
// 0 * 0), so the two kernels give the same bits.
#include <cuda_runtime.h>

#include <cstdint>

#include "heomgb_impl.cuh"
#include "stage.cuh"

namespace heomgb {

namespace {

__device__ __forceinline__ uint32_t sm_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp16(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sm_addr(dst_smem)), "l"(src_gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Shared memory of a CTA: H transposed and -H (real H, FP32), the -1 and +1
// coefficients per mode and case, the modes of every site, then two buffers
// of {stage input of `tile` ADOs at a padded ADO stride, their records, their
// ptr_p1 rows, their occupation rows}.  The 16-byte pad per ADO puts the same
// element of consecutive ADOs in different banks (the commutator's column
// reads).
struct SitesSmem {
  float* HT;     // n2: HT[c * n + a] = H[a][c]
  float* Hn;     // n2: Hn[c * n + b] = -H[c][b]
  float2* cm3;   // K * 3
  float2* cp2;   // K * 2
  int* sptr;     // n + 1
  int* smodes;   // K
  unsigned char* buf0;  // buffer b at buf0 + b * bsz (no array: a runtime index would put it in local memory)
  size_t bsz;
};
__host__ __device__ __forceinline__ int sites_ado_stride(int n2) { return n2 + 2; }  // float2 units
__host__ __device__ __forceinline__ size_t sites_head_bytes(int n, int K) {
  const size_t n2 = static_cast<size_t>(n) * n;
  return (sizeof(float) * 2 * n2 + sizeof(float2) * 5 * static_cast<size_t>(K) +
          sizeof(int) * (static_cast<size_t>(n) + 1 + K) + 15) & ~size_t(15);
}
__host__ __device__ __forceinline__ size_t sites_buf_bytes(int n, int K, int tile, int w) {
  return sizeof(float2) * static_cast<size_t>(tile) * sites_ado_stride(n * n) +
         sizeof(int4) * static_cast<size_t>(tile) * (1 + w) + 2 * sizeof(int) * static_cast<size_t>(tile) * K;
}
__device__ __forceinline__ SitesSmem sites_layout(unsigned char* raw, int n, int K, int tile, int w) {
  SitesSmem L;
  const int n2 = n * n;
  L.HT = reinterpret_cast<float*>(raw);
  L.Hn = L.HT + n2;
  L.cm3 = reinterpret_cast<float2*>(L.Hn + n2);
  L.cp2 = L.cm3 + 3 * K;
  L.sptr = reinterpret_cast<int*>(L.cp2 + 2 * K);
  L.smodes = L.sptr + n + 1;
  L.buf0 = raw + sites_head_bytes(n, K);
  L.bsz = sites_buf_bytes(n, K, tile, w);
  return L;
}

// Issues the cp.async copies of tile t (ADOs l0 .. l0+nt-1) into buffer b.
__device__ __forceinline__ void sites_stage(const DiagInst& I, const float2* y, int tile, int l0, int nt,
                                            unsigned char* b) {
  const int n2 = I.n2, K = I.K, w1 = 1 + I.site_w, sy = sites_ado_stride(n2), half = n2 / 2;
  float2* yt = reinterpret_cast<float2*>(b);
  int4* rec = reinterpret_cast<int4*>(yt + static_cast<size_t>(tile) * sy);
  int* p1s = reinterpret_cast<int*>(rec + static_cast<size_t>(tile) * w1);
  int* nks = p1s + static_cast<size_t>(tile) * K;
  const int ny = nt * half;  // 16-byte chunks of stage input (n2 is a multiple of 16)
  const float2* ysrc = y + static_cast<size_t>(l0) * n2;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) {
    const int lt = i / half, r = i - lt * half;
    cp16(yt + static_cast<size_t>(lt) * sy + 2 * r, ysrc + 2 * i);
  }
  const int nr = nt * w1;
  const int4* rsrc = I.site_rec + static_cast<size_t>(l0) * w1;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) cp16(rec + i, rsrc + i);
  const int nk = nt * K / 4;  // K is a multiple of 4
  const int* psrc = I.p1 + static_cast<size_t>(l0) * K;
  const int* nsrc = I.nidx + static_cast<size_t>(l0) * K;
  for (int i = threadIdx.x; i < nk; i += blockDim.x) {
    cp16(p1s + 4 * i, psrc + 4 * i);
    cp16(nks + 4 * i, nsrc + 4 * i);
  }
}

__device__ __forceinline__ float2 f4lo(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 f4hi(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float f4at(float4 v, int j) { return j == 0 ? v.x : j == 1 ? v.y : j == 2 ? v.z : v.w; }

// Real H.  A thread owns an RT x 4 block of one ADO (rows a0..a0+RT-1,
// columns b0..b0+3; RT = 4 or 2): per c it reads H[a0+i][c] (a row of H^T),
// -H[c][b0+j], four elements of row c and RT of column c of the ADO, and
// updates 4 RT complex accumulators with 8 RT paired FMAs.  Then, row by row,
// it adds the damping and bath terms and runs the stage epilogue of its four
// elements of that row.  RT = 2 halves the registers (more resident warps)
// for 25 % more shared-memory reads per element.
template <int KIND, int RT, int MAXT, int MINB>
__global__ void __launch_bounds__(MAXT, MINB) k_rhs_sites(const DiagSet ds, const Stage st) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double dt;
  int cur;
  if (!stage_prologue<KIND>(st, dt, cur)) return;
  const DiagInst& I = ds.inst[0];
  const int n = I.n, n2 = I.n2, K = I.K, w = I.site_w, w1 = 1 + w, void_idx = I.nh;
  const int nb = n >> 2, nr = n / RT, sy = sites_ado_stride(n2);
  const int tile = ds.sites_tile;
  const bool sqn = I.sqrt_norm != 0;
  const float2* __restrict__ y = stage_input<float2>(st, cur);
  const SitesSmem L = sites_layout(smem_raw, n, K, tile, w);
  const int n_tiles = ds.n_tiles;
  int t = blockIdx.x;
  if (t < n_tiles) sites_stage(I, y, tile, t * tile, min(tile, I.nh - t * tile), L.buf0);
  cp_commit();
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    const int a = i / n, c = i - a * n;
    const float h = I.H_f[i].x;  // H[a][c]
    L.HT[c * n + a] = h;
    L.Hn[i] = -h;
  }
  for (int i = threadIdx.x; i < 3 * K; i += blockDim.x) L.cm3[i] = I.site_cm3[i];
  for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) L.cp2[i] = I.site_cp2[i];
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.sptr[i] = I.site_ptr[i];
  for (int i = threadIdx.x; i < K; i += blockDim.x) L.smodes[i] = I.site_modes[i];
  const float2* __restrict__ csd = I.c_sd_f;
  double local = 0.0;
  int bsel = 0;
  for (; t < n_tiles; t += gridDim.x) {
    const int tn = t + gridDim.x;
    if (tn < n_tiles) sites_stage(I, y, tile, tn * tile, min(tile, I.nh - tn * tile), L.buf0 + (bsel ^ 1) * L.bsz);
    cp_commit();
    cp_wait<1>();  // this tile's copies (the next tile's may still be in flight)
    __syncthreads();
    const int l0 = t * tile, nt = min(tile, I.nh - l0);
    const float2* yt = reinterpret_cast<const float2*>(L.buf0 + bsel * L.bsz);
    const int4* rec = reinterpret_cast<const int4*>(yt + static_cast<size_t>(tile) * sy);
    const int* p1s = reinterpret_cast<const int*>(rec + static_cast<size_t>(tile) * w1);
    const int* nks = p1s + static_cast<size_t>(tile) * K;
    const int nq = nt * nr * nb;
    for (int q = threadIdx.x; q < nq; q += blockDim.x) {
      // q = (A * nt + lt) * nb + B: the lanes of a warp mostly share A
      const int B = q % nb, r = q / nb, lt = r % nt, A = r / nt;
      const int a0 = A * RT, b0 = B << 2, l = l0 + lt;
      const float2* yl = yt + static_cast<size_t>(lt) * sy;
      // -i[H, rho]: acc = H rho - rho H, k_rhs_diag's order over c
      float2 acc[RT][4];
#pragma unroll
      for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll 2
      for (int c = 0; c < n; ++c) {
        float ha[RT];  // H[a0+i][c]
        if (RT == 4) {
          const float4 h = *reinterpret_cast<const float4*>(L.HT + c * n + a0);
          ha[0] = h.x; ha[1] = h.y; ha[RT > 2 ? 2 : 0] = h.z; ha[RT > 3 ? 3 : 0] = h.w;
        } else {
          const float2 h = *reinterpret_cast<const float2*>(L.HT + c * n + a0);
          ha[0] = h.x; ha[1] = h.y;
        }
        const float4 hb = *reinterpret_cast<const float4*>(L.Hn + c * n + b0);  // -H[c][b0+j]
        const float4 r01 = *reinterpret_cast<const float4*>(yl + c * n + b0);   // rho[c][b0], [b0+1]
        const float4 r23 = *reinterpret_cast<const float4*>(yl + c * n + b0 + 2);
        const float2 row[4] = {f4lo(r01), f4hi(r01), f4lo(r23), f4hi(r23)};
        float2 col[RT];
#pragma unroll
        for (int i = 0; i < RT; ++i) col[i] = yl[(a0 + i) * n + c];  // rho[a0+i][c]
#pragma unroll
        for (int i = 0; i < RT; ++i) {
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float hbj = f4at(hb, j);
            acc[i][j] = __ffma2_rn(make_float2(ha[i], ha[i]), row[j], acc[i][j]);
            acc[i][j] = __ffma2_rn(make_float2(hbj, hbj), col[i], acc[i][j]);
          }
        }
      }
      const int4 hdr = rec[lt * w1];  // {occupied modes, any +1 neighbour, ngd bits}
      const float2 gl = make_float2(__int_as_float(hdr.z), __int_as_float(hdr.w));
      const int* p1r = p1s + lt * K;
      const int* nkr = nks + lt * K;
#pragma unroll
      for (int i = 0; i < RT; ++i) {
        const int a = a0 + i, e0 = a * n + b0;
        const size_t g0 = static_cast<size_t>(l) * n2 + e0;
        EpiPre pre[4];  // the row's epilogue loads, in flight while its terms are added
#pragma unroll
        for (int j = 0; j < 4; ++j) pre[j] = epi_pre<float, KIND>(st, g0 + j, cur);
        float2 D[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) D[j] = make_float2(-acc[i][j].y, acc[i][j].x);
        // (sum_k n_k gamma_k + sum_u s_delta_u (v_a - v_b)^2) rho
        {
          const float4 s01 = __ldg(reinterpret_cast<const float4*>(csd + e0));
          const float4 s23 = __ldg(reinterpret_cast<const float4*>(csd + e0 + 2));
          const float4 y01 = *reinterpret_cast<const float4*>(yl + e0);
          const float4 y23 = *reinterpret_cast<const float4*>(yl + e0 + 2);
          const float2 sd[4] = {f4lo(s01), f4hi(s01), f4lo(s23), f4hi(s23)};
          const float2 yv[4] = {f4lo(y01), f4hi(y01), f4lo(y23), f4hi(y23)};
#pragma unroll
          for (int j = 0; j < 4; ++j) cfma(D[j], make_float2(gl.x + sd[j].x, gl.y + sd[j].y), yv[j]);
        }
        // +1 terms (ADOs below the deepest tier): the modes of site a (row case)
        // and of site b (column case) merged in increasing k, as each
        // element's list holds them; an element's gathers are issued together
        if (hdr.y) {
          const int pa0 = L.sptr[a], pa1 = L.sptr[a + 1];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const int b = b0 + j;
            if (b == a) continue;  // c_plus vanishes on the diagonal
            int pa = pa0, pb = L.sptr[b];
            const int pb1 = L.sptr[b + 1];
            while (pa < pa1 || pb < pb1) {
              float2 v[4], cf[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                v[u] = make_float2(0.f, 0.f);
                cf[u] = make_float2(0.f, 0.f);
                if (pa < pa1 || pb < pb1) {
                  const int ka = pa < pa1 ? L.smodes[pa] : 0x7fffffff, kb = pb < pb1 ? L.smodes[pb] : 0x7fffffff;
                  const bool ta = ka < kb;
                  const int k = ta ? ka : kb;
                  pa += ta ? 1 : 0;
                  pb += ta ? 0 : 1;
                  const int lp = p1r[k];
                  float2 c2 = L.cp2[2 * k + (ta ? 0 : 1)];
                  if (lp != void_idx && (c2.x != 0.f || c2.y != 0.f)) {
                    if (sqn) {
                      const float f = sqrtf(static_cast<float>(nkr[k] + 1));
                      c2 = make_float2(f * c2.x, f * c2.y);
                    }
                    cf[u] = c2;
                    v[u] = __ldg(y + static_cast<size_t>(lp) * n2 + e0 + j);
                  }
                }
              }
#pragma unroll
              for (int u = 0; u < 4; ++u)
                if (cf[u].x != 0.f || cf[u].y != 0.f) cfma(D[j], cf[u], v[u]);
            }
          }
        }
        // -1 terms: the ADO's occupied modes in increasing k; an element couples
        // to mode k when the mode's site is its row or its column
        for (int m = 0; m < hdr.x; ++m) {
          const int4 rr = rec[lt * w1 + 1 + m];  // k, ptr_m1, n_k, site
          const int s = rr.w;
          const bool rowc = s == a;
          const int jc = s - b0;
          if (!rowc && static_cast<unsigned>(jc) >= 4u) continue;
          const float nk = sqn ? sqrtf(static_cast<float>(rr.z)) : static_cast<float>(rr.z);
          const float2* __restrict__ src = y + static_cast<size_t>(rr.y) * n2 + e0;
          if (rowc) {
            const float2 cr = L.cm3[3 * rr.x], cdg = L.cm3[3 * rr.x + 2];
            const float4 v01 = __ldg(reinterpret_cast<const float4*>(src));
            const float4 v23 = __ldg(reinterpret_cast<const float4*>(src + 2));
            const float2 v[4] = {f4lo(v01), f4hi(v01), f4lo(v23), f4hi(v23)};
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const float2 cm = (j == jc) ? cdg : cr;
              if (cm.x != 0.f || cm.y != 0.f) cfma(D[j], make_float2(nk * cm.x, nk * cm.y), v[j]);
            }
          } else {
            const float2 cm = L.cm3[3 * rr.x + 1];
            if (cm.x != 0.f || cm.y != 0.f) {
              const float2 cf = make_float2(nk * cm.x, nk * cm.y);
              const float2 v = __ldg(src + jc);
#pragma unroll
              for (int j = 0; j < 4; ++j)
                if (j == jc) cfma(D[j], cf, v);
            }
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) local += epi_post<float, KIND>(st, g0 + j, D[j], dt, cur, pre[j]);
      }
    }
    __syncthreads();  // every thread is done with this buffer before the prefetch after next reuses it
    bsel ^= 1;
  }
  cp_wait<0>();
  if (KIND == EPI_DP7) dp7_finish(st, local, ds.total);
}

// one record row per ADO: header, then its occupied modes
__global__ void k_site_records(const DiagInst I, const int* msite, int4* rec) {
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= I.nh) return;
  const int K = I.K, w1 = 1 + I.site_w;
  int4* r = rec + static_cast<size_t>(l) * w1;
  int cnt = 0, plus = 0;
  for (int k = 0; k < K; ++k) {
    const int nk = I.nidx[static_cast<size_t>(l) * K + k];
    const int lm = I.m1[static_cast<size_t>(l) * K + k];
    if (I.p1[static_cast<size_t>(l) * K + k] != I.nh) plus = 1;
    if (nk > 0 && lm != I.nh && cnt < I.site_w) r[1 + cnt++] = make_int4(k, lm, nk, msite[k]);
  }
  for (int j = cnt; j < I.site_w; ++j) r[1 + j] = make_int4(0, 0, 0, -1);
  const float2 g = I.ngd_f[l];
  r[0] = make_int4(cnt, plus, __float_as_int(g.x), __float_as_int(g.y));
}

// Kernel variants: (rows per register block, CTA size bound, resident CTAs):
// 4 rows at 128 registers (2 CTAs of 256), 2 rows at 80 (3 of 256), 64 (4 of 256)
// or 85 (2 of 384) registers.
template <int KIND>
cudaError_t launch_kind(const DiagSet& ds, const Stage& st, int grid, int block, cudaStream_t s) {
  void (*kern)(const DiagSet, const Stage);
  if (ds.sites_rt == 4)
    kern = k_rhs_sites<KIND, 4, 256, 2>;
  else if (ds.sites_minb == 3)
    kern = k_rhs_sites<KIND, 2, 256, 3>;
  else if (ds.sites_minb == 4)
    kern = k_rhs_sites<KIND, 2, 256, 4>;
  else
    kern = k_rhs_sites<KIND, 2, 384, 2>;
  if (ds.smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(ds.smem));
    if (e != cudaSuccess) return e;
  }
  kern<<<grid, block, ds.smem, s>>>(ds, st);
  return cudaGetLastError();
}

}  // namespace

bool sites_eligible(const DiagInst& I, bool mixed) {
  return mixed && I.site_local && I.site_rec && I.h_real && I.n >= 8 && (I.n & 3) == 0 && (I.K & 3) == 0 &&
         !I.term_p;
}

size_t sites_smem(int n, int K, int tile, int w) { return sites_head_bytes(n, K) + 2 * sites_buf_bytes(n, K, tile, w); }

bool sites_variant(int rt, int minb, int block) {
  if (rt == 4) return minb == 2 && block <= 256;
  if (rt != 2) return false;
  if (minb == 3 || minb == 4) return block <= 256;
  return minb == 2 && block > 256 && block <= 384;
}

cudaError_t launch_site_records(const DiagInst& I, const int* msite, int4* rec, cudaStream_t s) {
  if (I.nh <= 0) return cudaSuccess;
  k_site_records<<<(I.nh + 255) / 256, 256, 0, s>>>(I, msite, rec);
  ++g_launches;
  return cudaGetLastError();
}

cudaError_t launch_sites(const DiagSet& ds, const Stage& st, int grid, int block, cudaStream_t s) {
  cudaError_t e;
  switch (st.kind) {
    case EPI_RK4_1: e = launch_kind<EPI_RK4_1>(ds, st, grid, block, s); break;
    case EPI_RK4_2: e = launch_kind<EPI_RK4_2>(ds, st, grid, block, s); break;
    case EPI_RK4_3: e = launch_kind<EPI_RK4_3>(ds, st, grid, block, s); break;
    case EPI_RK4_4: e = launch_kind<EPI_RK4_4>(ds, st, grid, block, s); break;
    case EPI_LS: e = launch_kind<EPI_LS>(ds, st, grid, block, s); break;
    case EPI_DP: e = launch_kind<EPI_DP>(ds, st, grid, block, s); break;
    case EPI_DP7: e = launch_kind<EPI_DP7>(ds, st, grid, block, s); break;
    default: return cudaErrorInvalidValue;  // calc_diff (EPI_DIFF) keeps k_rhs_diag
  }
  ++g_launches;
  return e;
}

}  // namespace heomgb
