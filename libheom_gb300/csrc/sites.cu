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
// * A thread owns four consecutive elements of one row (a 1 x 4 micro-tile):
//   the commutator -i[H, rho] accumulates in registers with paired FP32 FMAs
//   (__ffma2_rn: both components of a complex value in one instruction) from
//   H and the tile's stage input in shared memory, and the thread then adds
//   the damping and bath terms and runs the stage epilogue for the same four
//   elements: no shared-memory round trip for the commutators.
// * The stage epilogue is a template argument (one instance per epilogue
//   kind), so no kind switch runs per element.
// * Tiles of consecutive ADOs are staged with cp.async (16-byte copies) into
//   two alternating shared-memory buffers: the next tile's stage input and
//   records are in flight while the current tile computes.
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

// acc += a * b for complex a, b, the component order of cfma (x: a.x b.x then
// -a.y b.y; y: a.x b.y then a.y b.x) in two paired FMAs
__device__ __forceinline__ void cfma2(float2& acc, float2 a, float2 b) {
  acc = __ffma2_rn(make_float2(a.x, a.x), b, acc);
  acc = __ffma2_rn(make_float2(-a.y, a.y), make_float2(b.y, b.x), acc);
}

// Shared memory of a CTA: H twice as (h, h) pairs (real H: H and -H; complex
// H: H as float2 in the first), the -1 coefficients, then two buffers of
// {stage input of `tile` ADOs, their records}.
struct SitesSmem {
  float2* Hp;   // n2: (h_ab, h_ab) (real H) or h_ab (complex H)
  float2* Hn;   // n2: (-h_ab, -h_ab) (real H)
  float2* cm3;  // K * 3
  unsigned char* buf0;  // buffer b at buf0 + b * bsz (no array: a runtime index would put it in local memory)
  size_t bsz;
};
__device__ __forceinline__ SitesSmem sites_layout(unsigned char* raw, int n2, int K, int tile, int w) {
  SitesSmem L;
  L.Hp = reinterpret_cast<float2*>(raw);
  L.Hn = L.Hp + n2;
  L.cm3 = L.Hn + n2;
  size_t off = (sizeof(float2) * (2 * static_cast<size_t>(n2) + 3 * static_cast<size_t>(K)) + 15) & ~size_t(15);
  const size_t bsz = sizeof(float2) * static_cast<size_t>(tile) * n2 + sizeof(int4) * static_cast<size_t>(tile) * (1 + w);
  L.buf0 = raw + off;
  L.bsz = bsz;
  return L;
}

// Issues the cp.async copies of tile t (ADOs l0 .. l0+nt-1) into buffer b.
__device__ __forceinline__ void sites_stage(const DiagInst& I, const float2* y, int tile, int l0, int nt,
                                            unsigned char* b) {
  const int n2 = I.n2, w1 = 1 + I.site_w;
  float2* yt = reinterpret_cast<float2*>(b);
  int4* rec = reinterpret_cast<int4*>(yt + static_cast<size_t>(tile) * n2);
  const int ny = nt * n2 / 2;  // 16-byte chunks of stage input (n2 is a multiple of 16)
  const float2* ysrc = y + static_cast<size_t>(l0) * n2;
  for (int i = threadIdx.x; i < ny; i += blockDim.x) cp16(yt + 2 * i, ysrc + 2 * i);
  const int nr = nt * w1;
  const int4* rsrc = I.site_rec + static_cast<size_t>(l0) * w1;
  for (int i = threadIdx.x; i < nr; i += blockDim.x) cp16(rec + i, rsrc + i);
}

template <int KIND, bool HREAL, int MINB>
__global__ void __launch_bounds__(256, MINB) k_rhs_sites(const DiagSet ds, const Stage st_in) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const Stage& st = st_in;  // its kind is KIND (a compile-time epilogue)
  double dt;
  int cur;
  if (!stage_prologue<KIND>(st, dt, cur)) return;
  const DiagInst& I = ds.inst[0];
  const int n = I.n, n2 = I.n2, K = I.K, w = I.site_w, w1 = 1 + w, void_idx = I.nh;
  const int tile = ds.sites_tile;
  const bool sqn = I.sqrt_norm != 0;
  const float2* __restrict__ y = stage_input<float2>(st, cur);
  const SitesSmem L = sites_layout(smem_raw, n2, K, tile, w);
  const int n_tiles = ds.n_tiles;
  int t = blockIdx.x;
  if (t < n_tiles) sites_stage(I, y, tile, t * tile, min(tile, I.nh - t * tile), L.buf0);
  cp_commit();
  for (int i = threadIdx.x; i < n2; i += blockDim.x) {
    const float2 h = I.H_f[i];
    if (HREAL) {
      L.Hp[i] = make_float2(h.x, h.x);
      L.Hn[i] = make_float2(-h.x, -h.x);
    } else {
      L.Hp[i] = h;
    }
  }
  for (int i = threadIdx.x; i < 3 * K; i += blockDim.x) L.cm3[i] = I.site_cm3[i];
  const int* __restrict__ plus_ptr = I.plus_ptr;
  const int* __restrict__ plus_mode = I.plus_mode;
  const float2* __restrict__ cpl = I.c_plus_f;
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
    const int4* rec = reinterpret_cast<const int4*>(yt + static_cast<size_t>(tile) * n2);
    const int ng = (nt * n2) >> 2;
    for (int q = threadIdx.x; q < ng; q += blockDim.x) {
      const int i0 = q << 2;
      const int lt = i0 / n2;
      const int e0 = i0 - lt * n2;
      const int a = e0 / n, b0 = e0 - a * n;
      const int l = l0 + lt;
      const size_t g0 = static_cast<size_t>(l) * n2 + e0;
      // the epilogue's loads first, so that they overlap the right-hand side
      EpiPre pre[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) pre[j] = epi_pre<float, KIND>(st, g0 + j, cur);
      const float2* yl = yt + static_cast<size_t>(lt) * n2;
      // -i[H, rho] (commutator), k_rhs_diag's order over c
      float2 acc[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) acc[j] = make_float2(0.f, 0.f);
      if (HREAL) {
#pragma unroll 4
        for (int c = 0; c < n; ++c) {
          const float2 hac = L.Hp[a * n + c];
          const float2 yac = yl[a * n + c];
          const float4 y01 = *reinterpret_cast<const float4*>(yl + c * n + b0);
          const float4 y23 = *reinterpret_cast<const float4*>(yl + c * n + b0 + 2);
          const float4 h01 = *reinterpret_cast<const float4*>(L.Hn + c * n + b0);
          const float4 h23 = *reinterpret_cast<const float4*>(L.Hn + c * n + b0 + 2);
          acc[0] = __ffma2_rn(hac, make_float2(y01.x, y01.y), acc[0]);
          acc[0] = __ffma2_rn(make_float2(h01.x, h01.y), yac, acc[0]);
          acc[1] = __ffma2_rn(hac, make_float2(y01.z, y01.w), acc[1]);
          acc[1] = __ffma2_rn(make_float2(h01.z, h01.w), yac, acc[1]);
          acc[2] = __ffma2_rn(hac, make_float2(y23.x, y23.y), acc[2]);
          acc[2] = __ffma2_rn(make_float2(h23.x, h23.y), yac, acc[2]);
          acc[3] = __ffma2_rn(hac, make_float2(y23.z, y23.w), acc[3]);
          acc[3] = __ffma2_rn(make_float2(h23.z, h23.w), yac, acc[3]);
        }
      } else {
        float2 neg[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) neg[j] = make_float2(0.f, 0.f);
#pragma unroll 2
        for (int c = 0; c < n; ++c) {
          const float2 hac = L.Hp[a * n + c];
          const float2 yac = yl[a * n + c];
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            cfma2(acc[j], hac, yl[c * n + b0 + j]);
            cfma2(neg[j], yac, L.Hp[c * n + b0 + j]);
          }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[j] = make_float2(acc[j].x - neg[j].x, acc[j].y - neg[j].y);
      }
      float2 D[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) D[j] = make_float2(-acc[j].y, acc[j].x);
      // (sum_k n_k gamma_k + sum_u s_delta_u (v_a - v_b)^2) rho
      const int4 hdr = rec[lt * w1];
      const float2 gl = make_float2(__int_as_float(hdr.z), __int_as_float(hdr.w));
      {
        const float4 s01 = __ldg(reinterpret_cast<const float4*>(csd + e0));
        const float4 s23 = __ldg(reinterpret_cast<const float4*>(csd + e0 + 2));
        const float2 sd[4] = {make_float2(s01.x, s01.y), make_float2(s01.z, s01.w), make_float2(s23.x, s23.y),
                              make_float2(s23.z, s23.w)};
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(D[j], make_float2(gl.x + sd[j].x, gl.y + sd[j].y), yl[e0 + j]);
      }
      // +1 terms (ADOs below the deepest tier), in each element's list order
      if (hdr.y) {
        const int* __restrict__ p1row = I.p1 + static_cast<size_t>(l) * K;
        const int* __restrict__ nrow = I.nidx + static_cast<size_t>(l) * K;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int e = e0 + j;
          const int pb = __ldg(plus_ptr + e), pe = __ldg(plus_ptr + e + 1);
          for (int p = pb; p < pe; ++p) {
            const int k = __ldg(plus_mode + p);
            const int lp = __ldg(p1row + k);
            if (lp == void_idx) continue;
            float2 cf = __ldg(cpl + p);
            if (sqn) {
              const float f = sqrtf(static_cast<float>(__ldg(nrow + k) + 1));
              cf = make_float2(f * cf.x, f * cf.y);
            }
            cfma(D[j], cf, __ldg(y + static_cast<size_t>(lp) * n2 + e));
          }
        }
      }
      // -1 terms: the ADO's occupied modes in increasing k; an element couples
      // to mode k when the mode's site is its row or its column
      for (int m = 0; m < hdr.x; ++m) {
        const int4 r = rec[lt * w1 + 1 + m];  // k, ptr_m1, n_k, site
        const int s = r.w;
        const bool row = s == a;
        const int jc = s - b0;
        if (!row && static_cast<unsigned>(jc) >= 4u) continue;
        const float nk = sqn ? sqrtf(static_cast<float>(r.z)) : static_cast<float>(r.z);
        const float2* __restrict__ src = y + static_cast<size_t>(r.y) * n2 + e0;
        if (row) {
          const float2 cr = L.cm3[3 * r.x], cd = L.cm3[3 * r.x + 2];
          const float4 v01 = __ldg(reinterpret_cast<const float4*>(src));
          const float4 v23 = __ldg(reinterpret_cast<const float4*>(src + 2));
          const float2 v[4] = {make_float2(v01.x, v01.y), make_float2(v01.z, v01.w), make_float2(v23.x, v23.y),
                               make_float2(v23.z, v23.w)};
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const float2 cm = (j == jc) ? cd : cr;
            if (cm.x != 0.f || cm.y != 0.f) cfma(D[j], make_float2(nk * cm.x, nk * cm.y), v[j]);
          }
        } else {
          const float2 cm = L.cm3[3 * r.x + 1];
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
    __syncthreads();  // every thread is done with this buffer before the prefetch after next reuses it
    bsel ^= 1;
  }
  cp_wait<0>();
  if (KIND == EPI_DP7) dp7_finish(st_in, local, ds.total);
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

template <int KIND>
cudaError_t launch_kind(const DiagSet& ds, const Stage& st, int grid, int block, cudaStream_t s) {
  void (*kern)(const DiagSet, const Stage);
  if (ds.sites_hreal)
    kern = ds.sites_minb == 3 ? k_rhs_sites<KIND, true, 3> : k_rhs_sites<KIND, true, 2>;
  else
    kern = ds.sites_minb == 3 ? k_rhs_sites<KIND, false, 3> : k_rhs_sites<KIND, false, 2>;
  if (ds.smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(ds.smem));
    if (e != cudaSuccess) return e;
  }
  kern<<<grid, block, ds.smem, s>>>(ds, st);
  return cudaGetLastError();
}

}  // namespace

bool sites_eligible(const DiagInst& I, bool mixed) {
  return mixed && I.site_local && I.site_rec && I.n >= 8 && (I.n & 3) == 0 && !I.term_p;
}

size_t sites_smem(int n2, int K, int tile, int w) {
  const size_t head = (sizeof(float2) * (2 * static_cast<size_t>(n2) + 3 * static_cast<size_t>(K)) + 15) & ~size_t(15);
  const size_t bsz = sizeof(float2) * static_cast<size_t>(tile) * n2 + sizeof(int4) * static_cast<size_t>(tile) * (1 + w);
  return head + 2 * bsz;
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
    case EPI_DIFF: e = launch_kind<EPI_DIFF>(ds, st, grid, block, s); break;
    case EPI_RK4_1: e = launch_kind<EPI_RK4_1>(ds, st, grid, block, s); break;
    case EPI_RK4_2: e = launch_kind<EPI_RK4_2>(ds, st, grid, block, s); break;
    case EPI_RK4_3: e = launch_kind<EPI_RK4_3>(ds, st, grid, block, s); break;
    case EPI_RK4_4: e = launch_kind<EPI_RK4_4>(ds, st, grid, block, s); break;
    case EPI_LS: e = launch_kind<EPI_LS>(ds, st, grid, block, s); break;
    case EPI_DP: e = launch_kind<EPI_DP>(ds, st, grid, block, s); break;
    case EPI_DP7: e = launch_kind<EPI_DP7>(ds, st, grid, block, s); break;
    default: return cudaErrorInvalidValue;
  }
  ++g_launches;
  return e;
}

}  // namespace heomgb
