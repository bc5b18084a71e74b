// The FP64 form's Dormand-Prince output interval in one cooperative launch
// (k_dp_resident64): rkdp::solve_adaptive_step (rkdp.h:81-179) with the
// right-hand side of heom_hilb::calc_diff_impl (heom_hilb.h:70-215) for
// site-local baths (every V_u diagonal with a single nonzero entry).
//
// CTA b owns ADOs b, b + G, b + 2G, ... (G CTAs; the same mix of tiers in
// every CTA).  It keeps their two FP64 states
// (current and candidate), the six stage vectors k_1..k_6 and two stage-input
// copies in shared memory, with the ADOs' records (occupied modes with their
// -1 neighbours), ptr_p1 and occupation rows and the per-mode coefficient
// tables; only the stage inputs the neighbours gather (and the candidate
// state) go through global memory.  Per stage, a thread computes the own part
// of each of its elements (commutator from the CTA's copy, damping), waits on
// the grid barrier for the other CTAs' previous stage, gathers only the
// neighbours its elements couple to (a -1 term per occupied mode of the ADO
// whose site is the element's row or column; +1 terms on ADOs below the
// deepest tier, the two sites' modes merged in increasing k) and runs the
// stage epilogue.  The arithmetic and its order are the FP64 stage kernels'
// (k_rhs_diag<double> with the EPI_DP / EPI_DP7 epilogues: explicit FMAs, the
// same coefficient products), so the first attempt's state is bit-identical
// to theirs; the error norm is summed per CTA and the partials are added in
// CTA order by every CTA, which runs the reference's FP64 step controller on
// its own copy of the controller state.
#include <cuda_runtime.h>

#include <cstdint>

#include "heomgb_impl.cuh"
#include "stage.cuh"

namespace heomgb {

namespace {

struct Res64Smem {
  double2* H;      // n2
  double2* S;      // 2 E: current and candidate state
  double2* K;      // 6 E: k_1..k_6
  double2* X;      // 2 E: stage-input copies
  double2* cm3;    // K * 3: -1 coefficients (row, column, diagonal case)
  double2* cp2;    // K * 2: +1 coefficients (row, column case)
  int4* rec;       // ados * (1 + w)
  int* p1;         // ados * K
  int* nk;         // ados * K
  int* sptr;       // n + 1
  int* smodes;     // K
};

__host__ __device__ __forceinline__ size_t res64_bytes(int n, int K, int w, int ados) {
  const size_t n2 = static_cast<size_t>(n) * n, E = n2 * ados;
  return sizeof(double2) * (n2 + 10 * E + 5 * static_cast<size_t>(K)) + sizeof(int4) * static_cast<size_t>(ados) * (1 + w) +
         sizeof(int) * (2 * static_cast<size_t>(ados) * K + n + 1 + K);
}

__device__ __forceinline__ Res64Smem res64_layout(unsigned char* raw, int n, int K, int w, int ados) {
  Res64Smem L;
  const size_t n2 = static_cast<size_t>(n) * n, E = n2 * ados;
  L.H = reinterpret_cast<double2*>(raw);
  L.S = L.H + n2;
  L.K = L.S + 2 * E;
  L.X = L.K + 6 * E;
  L.cm3 = L.X + 2 * E;
  L.cp2 = L.cm3 + 3 * K;
  L.rec = reinterpret_cast<int4*>(L.cp2 + 2 * K);
  L.p1 = reinterpret_cast<int*>(L.rec + static_cast<size_t>(ados) * (1 + w));
  L.nk = L.p1 + static_cast<size_t>(ados) * K;
  L.sptr = L.nk + static_cast<size_t>(ados) * K;
  L.smodes = L.sptr + n + 1;
  return L;
}

// c != 0 tested on the bit patterns (integer operations: this part's FP64
// pipe is the bottleneck of the FP64 form); -0 counts as zero
__device__ __forceinline__ bool nonzero(double2 c) {
  return ((static_cast<unsigned long long>(__double_as_longlong(c.x)) |
           static_cast<unsigned long long>(__double_as_longlong(c.y))) << 1) != 0ull;
}

// The terms of element e = (a, b) of CTA-local ADO lt, k_rhs_diag<double>'s
// order (+1 terms in increasing k, then -1 terms in increasing k), in batches
// of four: a batch's terms are formed, their gathers issued together, then
// added in order (the batch arrays are indexed only by unrolled positions, so
// they stay in registers).
__device__ __forceinline__ void res64_terms(const Res64Smem& L, const DiagInst& I, const double2* Xg, int lt, int a,
                                            int b, int e, int w1, double2& D) {
  const int K = I.K, n2 = I.n2, void_idx = I.nh;
  const bool sqn = I.sqrt_norm != 0;
  const int4 hdr = L.rec[lt * w1];
  if (hdr.y && a != b) {  // +1: c_plus vanishes on the diagonal
    const int* p1r = L.p1 + lt * K;
    int pa = L.sptr[a], pb = L.sptr[b];
    const int pa1 = L.sptr[a + 1], pb1 = L.sptr[b + 1];
    while (pa < pa1 || pb < pb1) {
      int off[4];
      double2 cf[4];
      bool val[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        val[u] = false;
        off[u] = 0;
        cf[u] = make_double2(0.0, 0.0);
        if (pa < pa1 || pb < pb1) {
          const int ka = pa < pa1 ? L.smodes[pa] : 0x7fffffff, kb = pb < pb1 ? L.smodes[pb] : 0x7fffffff;
          const bool ta = ka < kb;
          const int k = ta ? ka : kb;
          pa += ta ? 1 : 0;
          pb += ta ? 0 : 1;
          const int lp = p1r[k];
          double2 c = L.cp2[2 * k + (ta ? 0 : 1)];
          if (lp != void_idx && nonzero(c)) {
            if (sqn) {  // sqrt(n_k + 1) c_plus, as the set-up table forms it
              const double f = sqrt(static_cast<double>(L.nk[lt * K + k] + 1));
              c = make_double2(f * c.x, f * c.y);
            }
            off[u] = lp * n2 + e;
            cf[u] = c;
            val[u] = true;
          }
        }
      }
      double2 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = val[u] ? __ldcg(Xg + off[u]) : make_double2(0.0, 0.0);
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (val[u]) cfma(D, cf[u], v[u]);
    }
  }
  for (int m0 = 0; m0 < hdr.x; m0 += 4) {  // -1: the ADO's occupied modes
    int off[4];
    double2 cf[4];
    bool val[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      val[u] = false;
      off[u] = 0;
      cf[u] = make_double2(0.0, 0.0);
      if (m0 + u < hdr.x) {
        const int4 r = L.rec[lt * w1 + 1 + m0 + u];  // k, ptr_m1, n_k, site
        if (r.w == a || r.w == b) {
          const int cs = r.w == a ? (r.w == b ? 2 : 0) : 1;
          const double2 cm = L.cm3[3 * r.x + cs];
          if (nonzero(cm)) {
            const double f = sqn ? sqrt(static_cast<double>(r.z)) : occ<double>(r.z);
            off[u] = r.y * n2 + e;
            cf[u] = make_double2(f * cm.x, f * cm.y);
            val[u] = true;
          }
        }
      }
    }
    double2 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = val[u] ? __ldcg(Xg + off[u]) : make_double2(0.0, 0.0);
#pragma unroll
    for (int u = 0; u < 4; ++u)
      if (val[u]) cfma(D, cf[u], v[u]);
  }
}

template <bool HREAL, int EPT>
__global__ void __launch_bounds__(kResidentMaxBlock, 2) k_dp_resident64(const ResidentArgs R) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ DpCtl c;
  const DiagInst& I = R.inst;
  const int n = I.n, n2 = I.n2, K = I.K, w1 = 1 + I.site_w;
  // CTA b owns ADOs b, b + G, b + 2 G, ... (G CTAs): every CTA gets the same
  // mix of tiers (ADOs are ordered by tier, and only those below the deepest
  // have +1 terms), so no CTA holds up the grid barriers with more work
  const int G = gridDim.x, b0 = blockIdx.x;
  const int na = b0 < I.nh ? (I.nh - 1 - b0) / G + 1 : 0, E = na * n2;
  const Res64Smem L = res64_layout(smem_raw, n, K, I.site_w, R.ados_per_cta);
  double2* Yt0 = reinterpret_cast<double2*>(R.Ytmp[0]);  // stage inputs 2..6 (alternating; no array:
  double2* Yt1 = reinterpret_cast<double2*>(R.Ytmp[1]);  // a runtime index would put it in local memory)
  for (int i = threadIdx.x; i < n2; i += blockDim.x) L.H[i] = I.H[i];
  for (int i = threadIdx.x; i < 3 * K; i += blockDim.x) L.cm3[i] = I.site_cm3_d[i];
  for (int i = threadIdx.x; i < 2 * K; i += blockDim.x) L.cp2[i] = I.site_cp2_d[i];
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.sptr[i] = I.site_ptr[i];
  for (int i = threadIdx.x; i < K; i += blockDim.x) L.smodes[i] = I.site_modes[i];
  for (int i = threadIdx.x; i < na * w1; i += blockDim.x) {
    const int lt = i / w1;
    L.rec[i] = I.site_rec[static_cast<size_t>(b0 + lt * G) * w1 + (i - lt * w1)];
  }
  for (int i = threadIdx.x; i < na * K; i += blockDim.x) {
    const int lt = i / K;
    const size_t gi = static_cast<size_t>(b0 + lt * G) * K + (i - lt * K);
    L.p1[i] = I.p1[gi];
    L.nk[i] = I.nidx[gi];
  }
  if (threadIdx.x == 0) c = *R.ctl;
  __syncthreads();
  {
    const int cur = c.cur;
    for (int le = threadIdx.x; le < E; le += blockDim.x) {
      const int lt = le / n2;
      const double2 v = R.S[cur][static_cast<size_t>(b0 + lt * G) * n2 + (le - lt * n2)];
      L.S[static_cast<size_t>(cur) * E + le] = v;
      L.X[le] = v;
    }
  }
  // the thread's elements and their damping coefficients (ngamma + s_delta term, k_rhs_diag's sum)
  int el_lt[EPT], el_e[EPT], el_a[EPT], el_b[EPT], el_g[EPT];
  double2 gd[EPT];
#pragma unroll
  for (int r = 0; r < EPT; ++r) {
    const int le = threadIdx.x + r * blockDim.x;
    const int lec = le < E ? le : 0;
    const int lt = lec / n2, e = lec - lt * n2, a = e / n;
    const int l = min(b0 + lt * G, I.nh - 1);
    el_lt[r] = lt;
    el_e[r] = e;
    el_a[r] = a;
    el_b[r] = e - a * n;
    el_g[r] = l * n2 + e;  // the element's index in the state vector
    const double2 g0 = I.ngd[l], g1 = I.c_sd[e];
    gd[r] = make_double2(g0.x + g1.x, g0.y + g1.y);
  }
  __syncthreads();
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
    const double dt = c.dt, atol = c.atol, rtol = c.rtol;
    const int cur = c.cur;
    const double2* Sc = L.S + static_cast<size_t>(cur) * E;
    double2* Sn = L.S + static_cast<size_t>(1 - cur) * E;
    double local = 0.0;
    for (int s = 0; s < 7 && ok; ++s) {
      // stage input: own ADOs from shared memory, neighbours from global memory
      const double2* Xg = s == 0 ? R.S[cur] : (s < 6 ? (((s - 1) & 1) ? Yt1 : Yt0) : R.S[1 - cur]);
      const double2* Xs = L.X + static_cast<size_t>(s & 1) * E;
      double2* Xn = L.X + static_cast<size_t>((s + 1) & 1) * E;
      double2 D[EPT];
#pragma unroll
      for (int r = 0; r < EPT; ++r) {  // commutator and damping from this CTA's copy
        const int le = threadIdx.x + r * blockDim.x;
        D[r] = make_double2(0.0, 0.0);
        if (le >= E) continue;
        const int a = el_a[r], b = el_b[r];
        const double2* yl = Xs + static_cast<size_t>(el_lt[r]) * n2;
        double2 acc = make_double2(0.0, 0.0);
        if (HREAL) {
#pragma unroll 4
          for (int cc = 0; cc < n; ++cc) {
            const double hac = L.H[a * n + cc].x, hcb = L.H[cc * n + b].x;
            const double2 ycb = yl[cc * n + b], yac = yl[a * n + cc];
            acc.x = fma(hac, ycb.x, acc.x);
            acc.x = fma(-hcb, yac.x, acc.x);
            acc.y = fma(hac, ycb.y, acc.y);
            acc.y = fma(-hcb, yac.y, acc.y);
          }
        } else {
          double2 neg = make_double2(0.0, 0.0);
#pragma unroll 4
          for (int cc = 0; cc < n; ++cc) {
            cfma(acc, L.H[a * n + cc], yl[cc * n + b]);
            cfma(neg, yl[a * n + cc], L.H[cc * n + b]);
          }
          acc.x -= neg.x;
          acc.y -= neg.y;
        }
        double2 Dv = make_double2(-acc.y, acc.x);
        cfma(Dv, gd[r], yl[el_e[r]]);
        D[r] = Dv;
      }
      if (s > 0) {  // the other CTAs' stage input of the last stage
        ok = grid_wait(R.bar, gen, R.spin_limit);
        if (!ok) break;
      }
#pragma unroll
      for (int r = 0; r < EPT; ++r) {
        const int le = threadIdx.x + r * blockDim.x;
        if (le >= E) continue;
        res64_terms(L, I, Xg, el_lt[r], el_a[r], el_b[r], el_e[r], w1, D[r]);
        // stage epilogue: the FP64 form's EPI_DP / EPI_DP7 (epi_pre / epi_post), explicit FMAs
        const double2 k = make_double2(-dt * D[r].x, -dt * D[r].y);
        const int g = el_g[r];
        if (s < 6) {
          double2 y = Sc[le];
          for (int j = 0; j < s; ++j) {
            const double cj = c_dpA[s + 1][j];
            const double2 kj = L.K[static_cast<size_t>(j) * E + le];
            y.x = fma(cj, kj.x, y.x);
            y.y = fma(cj, kj.y, y.y);
          }
          L.K[static_cast<size_t>(s) * E + le] = k;
          const double cs = c_dpA[s + 1][s];
          y.x = fma(cs, k.x, y.x);
          y.y = fma(cs, k.y, y.y);
          Xn[le] = y;
          if (s < 5) {
            ((s & 1) ? Yt1 : Yt0)[g] = y;
          } else {  // the candidate state (also the stage-7 input)
            Sn[le] = y;
            R.S[1 - cur][g] = y;
          }
        } else {  // stage 7: e = sum_j E_j k_j, scaled squared error
          const double2 k0 = L.K[le];
          double2 ee = make_double2(c_dpE[0] * k0.x, c_dpE[0] * k0.y);
          for (int j = 1; j < 6; ++j) {
            const double2 kj = L.K[static_cast<size_t>(j) * E + le];
            ee.x = fma(c_dpE[j], kj.x, ee.x);
            ee.y = fma(c_dpE[j], kj.y, ee.y);
          }
          ee.x = fma(c_dpE[6], k.x, ee.x);
          ee.y = fma(c_dpE[6], k.y, ee.y);
          const double2 x1 = Sn[le], x2 = Sc[le];
          const double m = fmax(fma(x1.x, x1.x, x1.y * x1.y), fma(x2.x, x2.x, x2.y * x2.y));
          const double e2 = fma(ee.x, ee.x, ee.y * ee.y);
          const double sc = fma(rtol, sqrt(m), atol);
          local += e2 / (sc * sc);
        }
      }
      if (s < 6) grid_arrive(R.bar, R);
    }
    if (!ok) break;
    const double part = block_sum(local);
    if (threadIdx.x == 0) R.partials[blockIdx.x] = part;
    grid_arrive(R.bar, R);
    ok = grid_wait(R.bar, gen, R.spin_limit);
    if (!ok) break;
    double v = 0.0;
    for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += blockDim.x) v += __ldcg(R.partials + i);
    v = block_sum(v);
    if (threadIdx.x == 0) dp_control(&c, v, R.n_total, false);  // the reference's FP64 controller
    __syncthreads();
    // the next attempt's stage-1 input (own part): the current state
    const double2* Snow = L.S + static_cast<size_t>(c.cur) * E;
    for (int le = threadIdx.x; le < E; le += blockDim.x) L.X[le] = Snow[le];
    __syncthreads();
  }
  if (ok && blockIdx.x == 0 && threadIdx.x == 0) *R.ctl = c;
}

}  // namespace

size_t resident_dp64_smem(const DiagInst& I, int ados_per_cta) {
  return res64_bytes(I.n, I.K, I.site_w, ados_per_cta);
}

const void* resident_dp64_kernel(bool hreal, int ept) {
  if (ept == 1) return hreal ? reinterpret_cast<const void*>(k_dp_resident64<true, 1>)
                             : reinterpret_cast<const void*>(k_dp_resident64<false, 1>);
  if (ept == 2) return hreal ? reinterpret_cast<const void*>(k_dp_resident64<true, 2>)
                             : reinterpret_cast<const void*>(k_dp_resident64<false, 2>);
  return nullptr;
}

}  // namespace heomgb
