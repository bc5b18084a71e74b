// Stage kernel for site-local baths: every bath couples through a diagonal V_u
// with a single nonzero entry (the exciton aggregates, V_j = |j><j|), the
// state's n_state a multiple of 4 (n >= 8), mixed form (FP32 stage input,
// FP64 state).  Same operator and stage epilogues as k_rhs_diag
// (heom_hilb.h:96-215 with the fused rk4 / lsrk4 / rkdp stages), with the
// work of a tile of consecutive ADOs in three passes:
//
// 1. Commutator and damping: a thread owns an RT x 4 block of one ADO; -i[H,
//    rho] accumulates in registers with paired FP32 FMAs (__ffma2_rn: both
//    components of a complex value in one instruction) from H and the tile's
//    stage input in shared memory, the damping is added, and after a CTA
//    barrier the block replaces the stage input in shared memory.  Meanwhile
//    the -1 neighbours' values the tile needs are in flight into shared
//    memory (cp.async, issued at the start of the tile).
// 2. Bath terms, one warp per ADO.  Element (a, b) couples only to the modes
//    of the baths at sites a and b, so mode k (site s) touches row s and
//    column s of an ADO; lane x takes elements (s, x) and (x, s), which no
//    other lane touches for that mode, and the modes follow one another in
//    increasing k (__syncwarp), since a later mode of another site reaches
//    some of the same elements through other lanes.  First the +1 terms, only
//    on ADOs below the deepest tier (6 % of the 24-site hierarchy), their
//    gathers issued eight modes at a time; then the -1 terms over the ADO's
//    occupied modes (a per-ADO list built at set-up) from shared memory.
// 3. Stage epilogue: one element per thread over the tile's contiguous range
//    (coalesced), four elements' loads in flight per thread; the epilogue is a
//    template argument (one instance per epilogue kind).
//
// Tiles are staged with cp.async (16-byte copies) into two alternating
// shared-memory buffers: the next tile's stage input and records are in flight
// while the current tile computes.  A thread owns at most one register block
// per tile (the host admits only such shapes).
//
// Every element's arithmetic and its order are k_rhs_diag's (commutator over
// c, then the damping, the +1 terms in increasing k, the -1 terms in
// increasing k; terms with no neighbour are skipped, which the other kernels
// add as 0 * 0, which can only change the sign of a zero), so the two kernels
// give the same values.
#include <cuda_runtime.h>

#include <cstdint>

// The stage epilogues here round the new FP64 state to its FP32 copy with the
// hardware conversion: this kernel is issue-bound with its FP64 pipe mostly
// idle, and the hardware conversion takes 22 of its 295 instructions per
// element off the issue slots on the 24-site stage (258 against 260 µs).
#define HEOMGB_HW_D2F_EPILOGUE 1
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
__device__ __forceinline__ void cp8(void* dst_smem, const void* src_gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sm_addr(dst_smem)), "l"(src_gmem) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// Shared memory of a CTA: H transposed and -H (real H, FP32), the -1 and +1
// coefficients per mode and case, the modes of every site and the site of
// every mode, the tile's -1 neighbour values, then two buffers of {stage
// input of `tile` ADOs (then their right-hand sides), their records, their
// ptr_p1 rows, their occupation rows}.  ADOs sit at a padded stride (n^2 + 2 complex values), which puts the
// same element of consecutive ADOs in different banks.
struct SitesSmem {
  float* HT;     // n2: HT[c * n + a] = H[a][c]
  float* Hn;     // n2: Hn[c * n + b] = -H[c][b]
  float2* cm3;   // K * 3
  float2* cp2;   // K * 2
  int* sptr;     // n + 1
  int* smodes;   // K
  int* msite;    // K: the site of mode k
  float2* nb;    // tile * w * 2 * n: row s and column s of each -1 neighbour
  unsigned char* buf0;  // buffer b at buf0 + b * bsz (no array: a runtime index would put it in local memory)
  size_t bsz;
};
__host__ __device__ __forceinline__ int sites_ado_stride(int n2) { return n2 + 2; }  // float2 units
__host__ __device__ __forceinline__ size_t sites_head_bytes(int n, int K) {
  const size_t n2 = static_cast<size_t>(n) * n;
  return (sizeof(float) * 2 * n2 + sizeof(float2) * 5 * static_cast<size_t>(K) +
          sizeof(int) * (static_cast<size_t>(n) + 1 + 2 * static_cast<size_t>(K)) + 15) & ~size_t(15);
}
__host__ __device__ __forceinline__ size_t sites_nb_bytes(int n, int tile, int w) {
  return sizeof(float2) * static_cast<size_t>(tile) * w * 2 * n;
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
  L.msite = L.smodes + K;
  L.nb = reinterpret_cast<float2*>(raw + sites_head_bytes(n, K));
  L.buf0 = raw + sites_head_bytes(n, K) + sites_nb_bytes(n, tile, w);
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

// Real H.  Pass 1: a thread owns an RT x 4 block of one ADO (rows
// a0..a0+RT-1, columns b0..b0+3; RT = 4 or 2): per c it reads H[a0+i][c] (a
// row of H^T), -H[c][b0+j], four elements of row c and RT of column c of the
// ADO, and updates 4 RT complex accumulators with 8 RT paired FMAs; it adds
// the damping and stores the block.  RT = 2 halves the registers (more
// resident warps) for 25 % more shared-memory reads per element.
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
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
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
  for (int sidx = threadIdx.x; sidx < n; sidx += blockDim.x)
    for (int p = I.site_ptr[sidx]; p < I.site_ptr[sidx + 1]; ++p) L.msite[I.site_modes[p]] = sidx;
  const float2* __restrict__ csd = I.c_sd_f;
  double local = 0.0;
  int bsel = 0;
  for (; t < n_tiles; t += gridDim.x) {
    cp_wait<0>();  // this tile's stage input and records (issued a tile ago)
    __syncthreads();
    const int l0 = t * tile, nt = min(tile, I.nh - l0);
    float2* yt = reinterpret_cast<float2*>(L.buf0 + bsel * L.bsz);
    const int4* rec = reinterpret_cast<const int4*>(yt + static_cast<size_t>(tile) * sy);
    const int* p1s = reinterpret_cast<const int*>(rec + static_cast<size_t>(tile) * w1);
    const int* nks = p1s + static_cast<size_t>(tile) * K;
    // the -1 neighbours' row s and column s for every occupied mode of the
    // tile's ADOs (nb[((lt * w + m) * 2 + part) * n + x]), then the next tile
    for (int lt = warp; lt < nt; lt += nwarps) {
      const int nm = rec[lt * w1].x;
      for (int m = 0; m < nm; ++m) {
        const int4 rr = rec[lt * w1 + 1 + m];  // k, ptr_m1, n_k, site
        const float2* src = y + static_cast<size_t>(rr.y) * n2;
        float2* dst = L.nb + static_cast<size_t>((lt * w + m) * 2) * n;
        for (int x = lane; x < 2 * n; x += 32)
          cp8(dst + x, x < n ? src + rr.w * n + x : src + (x - n) * n + rr.w);
      }
    }
    cp_commit();
    const int tn = t + gridDim.x;
    if (tn < n_tiles) sites_stage(I, y, tile, tn * tile, min(tile, I.nh - tn * tile), L.buf0 + (bsel ^ 1) * L.bsz);
    cp_commit();
    // pass 1: commutator and damping; one register block per thread
    const int nq = nt * nr * nb;
    const int q = threadIdx.x;
    const int B = q % nb, rq = q / nb, lq = rq % nt, A = rq / nt;
    const int a0 = A * RT, b0 = B << 2;
    float2 D[RT][4];
    if (q < nq) {
      // q = (A * nt + lt) * nb + B: the lanes of a warp mostly share A
      const float2* yl = yt + static_cast<size_t>(lq) * sy;
      // -i[H, rho]: acc = H rho - rho H, k_rhs_diag's order over c
      float2 acc[RT][4];
#pragma unroll
      for (int i = 0; i < RT; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = make_float2(0.f, 0.f);
#pragma unroll 4
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
      const int4 hdr = rec[lq * w1];  // {occupied modes, any +1 neighbour, ngd bits}
      const float2 gl = make_float2(__int_as_float(hdr.z), __int_as_float(hdr.w));
#pragma unroll
      for (int i = 0; i < RT; ++i) {
        const int e0 = (a0 + i) * n + b0;
#pragma unroll
        for (int j = 0; j < 4; ++j) D[i][j] = make_float2(-acc[i][j].y, acc[i][j].x);
        // (sum_k n_k gamma_k + sum_u s_delta_u (v_a - v_b)^2) rho
        const float4 s01 = __ldg(reinterpret_cast<const float4*>(csd + e0));
        const float4 s23 = __ldg(reinterpret_cast<const float4*>(csd + e0 + 2));
        const float4 y01 = *reinterpret_cast<const float4*>(yl + e0);
        const float4 y23 = *reinterpret_cast<const float4*>(yl + e0 + 2);
        const float2 sd[4] = {f4lo(s01), f4hi(s01), f4lo(s23), f4hi(s23)};
        const float2 yv[4] = {f4lo(y01), f4hi(y01), f4lo(y23), f4hi(y23)};
#pragma unroll
        for (int j = 0; j < 4; ++j) cfma(D[i][j], make_float2(gl.x + sd[j].x, gl.y + sd[j].y), yv[j]);
      }
    }
    cp_wait<1>();  // the -1 neighbour values (the next tile's copies may still be in flight)
    __syncthreads();  // every thread has read the stage input: the right-hand sides replace it
    if (q < nq) {
      float2* dl = yt + static_cast<size_t>(lq) * sy;
#pragma unroll
      for (int i = 0; i < RT; ++i) {
        const int e0 = (a0 + i) * n + b0;
        *reinterpret_cast<float4*>(dl + e0) = make_float4(D[i][0].x, D[i][0].y, D[i][1].x, D[i][1].y);
        *reinterpret_cast<float4*>(dl + e0 + 2) = make_float4(D[i][2].x, D[i][2].y, D[i][3].x, D[i][3].y);
      }
    }
    __syncthreads();
    // pass 2: bath terms, one warp per ADO
    for (int lt = warp; lt < nt; lt += nwarps) {
      const int4 hdr = rec[lt * w1];
      float2* dl = yt + static_cast<size_t>(lt) * sy;
      if (hdr.y) {  // +1 terms in increasing k, eight modes' gathers at a time
        const int* p1r = p1s + lt * K;
        const int* nkr = nks + lt * K;
        for (int k0 = 0; k0 < K; k0 += 8) {
          float2 vr[8], vc[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int k = k0 + u;
            vr[u] = make_float2(0.f, 0.f);
            vc[u] = make_float2(0.f, 0.f);
            if (k < K && p1r[k] != void_idx && lane < n) {
              const int sk = L.msite[k];
              const float2* __restrict__ src = y + static_cast<size_t>(p1r[k]) * n2;
              if (lane != sk) {
                vr[u] = __ldg(src + sk * n + lane);
                vc[u] = __ldg(src + lane * n + sk);
              }
            }
          }
#pragma unroll
          for (int u = 0; u < 8; ++u) {
            const int k = k0 + u;
            if (k >= K) break;               // warp-uniform
            if (p1r[k] == void_idx) continue;  // warp-uniform
            const int sk = L.msite[k];
            float2 cr = L.cp2[2 * k], cc = L.cp2[2 * k + 1];  // row case (a = s), column case (b = s)
            const bool ur = cr.x != 0.f || cr.y != 0.f, uc = cc.x != 0.f || cc.y != 0.f;
            if (sqn) {
              const float f = sqrtf(static_cast<float>(nkr[k] + 1));
              cr = make_float2(f * cr.x, f * cr.y);
              cc = make_float2(f * cc.x, f * cc.y);
            }
            for (int x = lane; x < n; x += 32) {
              if (x == sk) continue;  // c_plus vanishes on the diagonal
              float2 a = vr[u], b = vc[u];
              if (x >= 32) {  // n > 32: the later columns' gathers here
                const float2* __restrict__ src = y + static_cast<size_t>(p1r[k]) * n2;
                a = __ldg(src + sk * n + x);
                b = __ldg(src + x * n + sk);
              }
              if (ur) cfma(dl[sk * n + x], cr, a);
              if (uc) cfma(dl[x * n + sk], cc, b);
            }
            __syncwarp();
          }
        }
      }
      // -1 terms: the ADO's occupied modes in increasing k, values from nb
      for (int m = 0; m < hdr.x; ++m) {
        const int4 rr = rec[lt * w1 + 1 + m];  // k, ptr_m1, n_k, site
        const int s = rr.w, k = rr.x;
        const float nk = sqn ? sqrtf(static_cast<float>(rr.z)) : static_cast<float>(rr.z);
        const float2 cr = L.cm3[3 * k], cc = L.cm3[3 * k + 1], cdg = L.cm3[3 * k + 2];
        const float2* vrow = L.nb + static_cast<size_t>((lt * w + m) * 2) * n;
        const float2* vcol = vrow + n;
        for (int x = lane; x < n; x += 32) {
          const float2 cm = x == s ? cdg : cr;
          if (cm.x != 0.f || cm.y != 0.f) cfma(dl[s * n + x], make_float2(nk * cm.x, nk * cm.y), vrow[x]);
          if (x != s && (cc.x != 0.f || cc.y != 0.f)) cfma(dl[x * n + s], make_float2(nk * cc.x, nk * cc.y), vcol[x]);
        }
        __syncwarp();
      }
    }
    __syncthreads();
    // pass 3: stage epilogue over the tile's elements (consecutive in the
    // state), four per thread in flight
    {
      const int ne = nt * n2;
      const size_t g0 = static_cast<size_t>(l0) * n2;
      int lt = 0, e = threadIdx.x;  // element threadIdx.x: ADO lt, offset e
      while (e >= n2 && lt < nt) {
        e -= n2;
        ++lt;
      }
      for (int idx = threadIdx.x; idx < ne; idx += 4 * blockDim.x) {
        EpiPre pre[4];
        float2 Dv[4];
        int ix[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          ix[u] = idx + u * blockDim.x;
          if (ix[u] < ne) {
            pre[u] = epi_pre<float, KIND>(st, g0 + ix[u], cur);
            Dv[u] = yt[static_cast<size_t>(lt) * sy + e];
          }
          e += blockDim.x;
          while (e >= n2) {
            e -= n2;
            ++lt;
          }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (ix[u] < ne) local += epi_post<float, KIND>(st, g0 + ix[u], Dv[u], dt, cur, pre[u]);
      }
    }
    __syncthreads();  // every thread is done with this buffer before it is refilled
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

size_t sites_smem(int n, int K, int tile, int w) {
  return sites_head_bytes(n, K) + sites_nb_bytes(n, tile, w) + 2 * sites_buf_bytes(n, K, tile, w);
}

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
