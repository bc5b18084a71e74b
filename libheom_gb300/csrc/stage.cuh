// Device helpers shared by the stage kernels of every translation unit:
// complex arithmetic, the Dormand-Prince tableau, the fused Runge-Kutta stage
// epilogues (epi_pre / epi_post), the stage-7 error-norm finish with the step
// controller, and the stage prologue.  Everything here is internal linkage
// (static or inline), so each kernel file holds its own copy.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <type_traits>

#include "heomgb_impl.cuh"
#include "fpconv.cuh"

namespace heomgb {

// ------------------------------------------------------------------ complex helpers
template <typename T> struct CT;
template <> struct CT<double> { using type = double2; };
template <> struct CT<float> { using type = float2; };
template <typename T> using cx_t = typename CT<T>::type;

template <typename T> __device__ __forceinline__ cx_t<T> cx(T re, T im);
template <> __device__ __forceinline__ double2 cx<double>(double re, double im) { return make_double2(re, im); }
template <> __device__ __forceinline__ float2 cx<float>(float re, float im) { return make_float2(re, im); }

template <typename TC> __device__ __forceinline__ cx_t<TC> ldc(const double2* p) {
  const double2 v = __ldg(p);
  return cx<TC>(static_cast<TC>(v.x), static_cast<TC>(v.y));
}
template <typename TC> __device__ __forceinline__ cx_t<TC> ldc(const float2* p) {
  const float2 v = __ldg(p);
  return cx<TC>(static_cast<TC>(v.x), static_cast<TC>(v.y));
}
// acc += a*b
template <typename C> __device__ __forceinline__ void cfma(C& acc, C a, C b) {
  acc.x = fma(a.x, b.x, acc.x);
  acc.x = fma(-a.y, b.y, acc.x);
  acc.y = fma(a.x, b.y, acc.y);
  acc.y = fma(a.y, b.x, acc.y);
}
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// A hierarchy occupation 0 <= v < 2^31 as TC.  For double the IEEE-754
// encoding is assembled with integer operations (exact, like the conversion
// instruction), which keeps it off this part's narrow FP64 pipe.
template <typename TC> __device__ __forceinline__ TC occ(int v);
template <> __device__ __forceinline__ float occ<float>(int v) { return static_cast<float>(v); }
template <> __device__ __forceinline__ double occ<double>(int v) {
  if (v <= 0) return 0.0;
  const int e = 31 - __clz(v);  // the leading bit; it moves to bit 52 of the significand
  const unsigned long long sig = static_cast<unsigned long long>(v) << (52 - e);
  return __longlong_as_double((static_cast<unsigned long long>(1023 + e) << 52) | (sig & ((1ull << 52) - 1)));
}
__device__ __forceinline__ double2 to_d(double2 v) { return v; }
__device__ __forceinline__ double2 to_d(float2 v) { return make_double2(f2d(v.x), f2d(v.y)); }
// FP64 -> FP32 of a complex value (round to nearest even).  The integer-
// assembled d2f keeps the FP64 pipe free; a translation unit whose kernels
// have that pipe to spare and are issue-bound defines
// HEOMGB_HW_D2F_EPILOGUE to take the hardware conversion instead (the same
// bits: both are the IEEE conversion).
__device__ __forceinline__ float2 to_f(double2 v) {
#if defined(HEOMGB_HW_D2F_EPILOGUE)
  return make_float2(__double2float_rn(v.x), __double2float_rn(v.y));
#else
  return make_float2(d2f(v.x), d2f(v.y));
#endif
}

template <typename TC> __device__ __forceinline__ const cx_t<TC>* pick(const double2* d, const float2* f);
template <> __device__ __forceinline__ const double2* pick<double>(const double2* d, const float2*) { return d; }
template <> __device__ __forceinline__ const float2* pick<float>(const double2*, const float2* f) { return f; }

// bulk-precision vector access: bulk is float2 in mixed mode, double2 otherwise
template <typename TC> __device__ __forceinline__ void st_bulk(void* base, size_t g, double2 v) {
  if constexpr (std::is_same<TC, double>::value) {
    static_cast<double2*>(base)[g] = v;
  } else {
    static_cast<float2*>(base)[g] = to_f(v);
  }
}
template <typename TC> __device__ __forceinline__ double2 ld_bulk(const void* base, size_t g) {
  if constexpr (std::is_same<TC, double>::value) {
    return static_cast<const double2*>(base)[g];
  } else {
    return to_d(static_cast<const float2*>(base)[g]);
  }
}
// Streaming (evict-first) variants for the epilogue's own vectors: they are
// touched once per stage, so they should not push the right-hand-side input,
// which every neighbour gather reads, out of L2.
template <typename TC> __device__ __forceinline__ void st_bulk_cs(void* base, size_t g, double2 v) {
  if constexpr (std::is_same<TC, double>::value) {
    __stcs(static_cast<double2*>(base) + g, v);
  } else {
    __stcs(static_cast<float2*>(base) + g, to_f(v));
  }
}
template <typename TC> __device__ __forceinline__ double2 ld_bulk_cs(const void* base, size_t g) {
  if constexpr (std::is_same<TC, double>::value) {
    return __ldcs(static_cast<const double2*>(base) + g);
  } else {
    return to_d(__ldcs(static_cast<const float2*>(base) + g));
  }
}
// value a bulk vector will hold after a store (rounding in mixed mode)
template <typename TC> __device__ __forceinline__ double2 as_bulk(double2 v) {
  if constexpr (std::is_same<TC, double>::value) {
    return v;
  } else {
    return to_d(to_f(v));
  }
}

// ------------------------------------------------------------------ Dormand-Prince tableau (rkdp.h:21-57)
static __constant__ double c_dpA[7][6] = {
    {0, 0, 0, 0, 0, 0},
    {1.0 / 5, 0, 0, 0, 0, 0},
    {3.0 / 40, 9.0 / 40, 0, 0, 0, 0},
    {44.0 / 45, -56.0 / 15, 32.0 / 9, 0, 0, 0},
    {19372.0 / 6561, -25360.0 / 2187, 64448.0 / 6561, -212.0 / 729, 0, 0},
    {9017.0 / 3168, -355.0 / 33, 46732.0 / 5247, 49.0 / 176, -5103.0 / 18656, 0},
    {35.0 / 384, 0, 500.0 / 1113, 125.0 / 192, -2187.0 / 6784, 11.0 / 84}};
static __constant__ double c_dpE[7] = {-71.0 / 57600, 0, 71.0 / 16695, -71.0 / 1920, 17253.0 / 339200, -22.0 / 525,
                                1.0 / 40};

// The mixed form's candidate state rho + sum_j B_j k_j (B = the last row of
// the tableau, k_j FP32) takes the sum as an unevaluated float pair hi + lo:
// each B_j is split into two floats (B_j = Bh_j + Bl_j to about 2^-48), each
// product's rounding error is recovered with an FMA and the additions use
// Knuth's TwoSum, so the pair carries the sum to about 2^-48 of sum |B_j k_j|;
// the FP64 state then takes hi and lo in two FP64 additions.  This replaces
// twelve FP64 FMAs and conversions per element, slow on this part, with FP32
// work of the same accuracy class.
#define HEOMGB_DP_B(j) (j == 0 ? 35.0 / 384 : j == 1 ? 0.0 : j == 2 ? 500.0 / 1113 : j == 3 ? 125.0 / 192 \
                        : j == 4 ? -2187.0 / 6784 : 11.0 / 84)
#define HEOMGB_SPLIT_LO(v) static_cast<float>((v) - static_cast<double>(static_cast<float>(v)))
static __constant__ float c_dpBh[6] = {static_cast<float>(HEOMGB_DP_B(0)), static_cast<float>(HEOMGB_DP_B(1)),
                                static_cast<float>(HEOMGB_DP_B(2)), static_cast<float>(HEOMGB_DP_B(3)),
                                static_cast<float>(HEOMGB_DP_B(4)), static_cast<float>(HEOMGB_DP_B(5))};
static __constant__ float c_dpBl[6] = {HEOMGB_SPLIT_LO(HEOMGB_DP_B(0)), HEOMGB_SPLIT_LO(HEOMGB_DP_B(1)),
                                HEOMGB_SPLIT_LO(HEOMGB_DP_B(2)), HEOMGB_SPLIT_LO(HEOMGB_DP_B(3)),
                                HEOMGB_SPLIT_LO(HEOMGB_DP_B(4)), HEOMGB_SPLIT_LO(HEOMGB_DP_B(5))};
#undef HEOMGB_SPLIT_LO
#undef HEOMGB_DP_B

// (hi, lo) += (bh + bl) * k; the rounded operations are explicit so that no
// contraction merges the product into the TwoSum
__device__ __forceinline__ void ff_add_prod(float& hi, float& lo, float bh, float bl, float k) {
  const float p = __fmul_rn(bh, k);
  const float pe = fmaf(bh, k, -p);
  const float s = __fadd_rn(hi, p);
  const float bb = __fsub_rn(s, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  hi = s;
  lo = __fadd_rn(lo, __fadd_rn(__fadd_rn(err, pe), __fmul_rn(bl, k)));
}

// ------------------------------------------------------------------ step control
// rkdp.h:150-177 and adaptive_step_size_solver.h:45-55, one thread.  The
// mixed form takes the step-size factor err^-0.2 in FP32 (`fast`): it only
// scales the next step, FP32 resolves it far below the form's own rounding,
// and an FP64 pow is thousands of cycles on this part's FP64 pipe, on the
// critical path between two attempts.  The FP64 form keeps the reference's
// FP64 pow, so its step sequence follows the reference's.
static __device__ void dp_control(DpCtl* c, double sumsq, long long n, bool fast) {
  const double err = sqrt(sumsq) / sqrt(static_cast<double>(n));
  c->err = err;
  c->attempts += 1;
  c->count += 1;
  const double fac = fast ? static_cast<double>(powf(static_cast<float>(err), -0.2f)) : pow(err, -0.2);
  if (err < 1.0) {
    c->t += c->dt;
    c->dt *= 0.9 * ((fac < 10.0) ? fac : 10.0);
    c->cur ^= 1;
    c->accepted += 1;
    c->count = 0;
    if (c->t >= c->t_bound) c->done = 1;
  } else {
    c->dt *= 0.9 * ((0.2 < fac) ? fac : 0.2);
    if (c->dt < 1e-16) c->dt = 1e-16;
    if (c->count >= 1000) {  // the 1001st attempt gives up (rkdp.h:98-102)
      c->t = c->t_bound;
      c->count = 0;
      c->done = 1;
    }
  }
  if (!c->done && c->t + c->dt > c->t_bound) c->dt = c->t_bound - c->t;
  if (!isfinite(c->dt) || !isfinite(c->t)) {
    c->status = 1;
    c->done = 1;
  }
}

// ------------------------------------------------------------------ fused stage epilogue
// D is the operator value of heom_hilb.h:96-353 at element g; every solver
// stage uses k = -dt*D (calc_diff_impl with alpha = dt, beta = 0).
//
// The epilogue is split in two: epi_pre reads everything the stage
// combination needs that does not depend on D (issued before the
// right-hand side so its loads overlap it), epi_post adds the k term and
// stores.  epi_post returns the element's squared scaled error for EPI_DP7,
// else 0.
//
// FP64 form (TC = double): the reference's operation order (rk4.h:40-65,
// lsrk4.h:32-47, rkdp.h:111-153).  Mixed form (TC = float): stage inputs of
// the next right-hand side are formed in FP32 from the bulk copy of the
// state; the state and the RK4 accumulator are accumulated in FP64, the LSRK4
// buffer (a +-1 combination of FP32 k's) is FP32 and added to the FP64 state
// in FP64, and the Dormand-Prince candidate state rho + sum_j B_j k_j adds
// the sum of the FP32 k_j, carried as a float pair to about 2^-48
// (ff_add_prod), to the FP64 state.  The error vector e = sum_j E_j k_j only
// steers the step size: it is combined from the FP32 k_j in FP32, while the
// error norm's sum over elements and the step controller are FP64.
struct EpiPre {
  double2 a;   // FP64 partial result (accumulator, base state, partial sum)
  double2 b;   // FP64 base state (RK4 in FP64 form, LSRK4)
  float2 f;    // FP32 partial result (mixed-form stage inputs; high part of the candidate's sum)
  float2 g;    // low part of the mixed-form Dormand-Prince candidate's sum
  double m;    // squared error scale (EPI_DP7)
};

// KIND >= 0 fixes the epilogue kind at compile time (st.kind is then not read).
template <typename TC, int KIND = -1>
__device__ __forceinline__ EpiPre epi_pre(const Stage& st, size_t g, int cur) {
  constexpr bool MIX = std::is_same<TC, float>::value;
  EpiPre p;
  p.a = make_double2(0.0, 0.0);
  p.b = make_double2(0.0, 0.0);
  p.f = make_float2(0.f, 0.f);
  p.g = make_float2(0.f, 0.f);
  p.m = 0.0;
  switch (KIND >= 0 ? KIND : st.kind) {
    case EPI_DIFF:
      if (!st.beta_zero) p.a = cmul(st.beta, st.out[g]);
      break;
    case EPI_RK4_1:
    case EPI_RK4_2:
    case EPI_RK4_3:
      p.a = (KIND >= 0 ? KIND : st.kind) == EPI_RK4_1 ? __ldcs(st.S[0] + g) : __ldcs(st.acc + g);
      if constexpr (MIX)
        p.f = static_cast<const float2*>(st.Yb[0])[g];
      else
        p.b = __ldcs(st.S[0] + g);
      break;
    case EPI_RK4_4:
      p.a = __ldcs(st.acc + g);
      break;
    case EPI_LS:
      if constexpr (MIX) {  // FP32 buffer (the first half of the buffer allocation)
        if (!st.ls_first) p.f = __ldcs(reinterpret_cast<const float2*>(st.acc) + g);
      } else {
        if (!st.ls_first) p.a = __ldcs(st.acc + g);
      }
      p.b = __ldcs(st.S[st.ls_in] + g);
      break;
    case EPI_DP: {
      const int s_ = st.dp_stage;
      if constexpr (MIX) {
        if (s_ < 5) {
          float2 y = static_cast<const float2*>(st.Yb[cur])[g];
          for (int j = 0; j < s_; ++j) {
            const float c = static_cast<float>(c_dpA[s_ + 1][j]);
            const float2 kj = __ldcs(static_cast<const float2*>(st.K[j]) + g);
            y.x = fmaf(c, kj.x, y.x);
            y.y = fmaf(c, kj.y, y.y);
          }
          p.f = y;
        } else {  // candidate state rho + sum_j B_j k_j: the sum as a float pair (c_dpBh)
          p.a = __ldcs(st.S[cur] + g);
          float2 hi = make_float2(0.f, 0.f), lo = make_float2(0.f, 0.f);
          for (int j = 0; j < 5; ++j) {
            const float2 kj = __ldcs(static_cast<const float2*>(st.K[j]) + g);
            ff_add_prod(hi.x, lo.x, c_dpBh[j], c_dpBl[j], kj.x);
            ff_add_prod(hi.y, lo.y, c_dpBh[j], c_dpBl[j], kj.y);
          }
          p.f = hi;
          p.g = lo;
        }
      } else {  // explicit FMAs, shared with k_dp_resident64
        double2 y = __ldcs(st.S[cur] + g);
        for (int j = 0; j < s_; ++j) {
          const double c = c_dpA[s_ + 1][j];
          const double2 kj = ld_bulk_cs<TC>(st.K[j], g);
          y.x = fma(c, kj.x, y.x);
          y.y = fma(c, kj.y, y.y);
        }
        p.a = y;
      }
      break;
    }
    case EPI_DP7: {
      if constexpr (MIX) {  // FP32 stage vectors: combine them in FP32
        float2 e = make_float2(0.f, 0.f);
        for (int j = 0; j < 6; ++j) {
          const float c = static_cast<float>(c_dpE[j]);
          const float2 kj = __ldcs(static_cast<const float2*>(st.K[j]) + g);
          e.x = fmaf(c, kj.x, e.x);
          e.y = fmaf(c, kj.y, e.y);
        }
        p.f = e;
      } else {
        const double2 k0 = ld_bulk_cs<TC>(st.K[0], g);
        double2 e = make_double2(c_dpE[0] * k0.x, c_dpE[0] * k0.y);
        for (int j = 1; j < 6; ++j) {
          const double2 kj = ld_bulk_cs<TC>(st.K[j], g);
          e.x = fma(c_dpE[j], kj.x, e.x);
          e.y = fma(c_dpE[j], kj.y, e.y);
        }
        p.a = e;
      }
      if constexpr (MIX) {  // scale from the bulk copies of both states
        const float2 x1 = static_cast<const float2*>(st.Yb[1 - cur])[g];
        const float2 x2 = static_cast<const float2*>(st.Yb[cur])[g];
        p.m = f2d(fmaxf(x1.x * x1.x + x1.y * x1.y, x2.x * x2.x + x2.y * x2.y));
      } else {
        const double2 x1 = __ldcs(st.S[1 - cur] + g);
        const double2 x2 = __ldcs(st.S[cur] + g);
        p.m = fmax(fma(x1.x, x1.x, x1.y * x1.y), fma(x2.x, x2.x, x2.y * x2.y));
      }
      break;
    }
    default:
      break;
  }
  return p;
}

template <typename TC, int KIND = -1>
__device__ __forceinline__ double epi_post(const Stage& st, size_t g, cx_t<TC> Dc, double dt, int cur,
                                           const EpiPre& p) {
  constexpr bool MIX = std::is_same<TC, float>::value;
  // the mixed form's stage epilogues take the FP32 value; only calc_diff
  // (EPI_DIFF) and the FP64 form need it in FP64
  const double2 D = (MIX && (KIND >= 0 ? KIND : st.kind) != EPI_DIFF) ? make_double2(0.0, 0.0) : to_d(Dc);
  switch (KIND >= 0 ? KIND : st.kind) {
    case EPI_DIFF: {
      const double2 ad = cmul(st.alpha, D);
      st.out[g] = make_double2(p.a.x - ad.x, p.a.y - ad.y);
      return 0.0;
    }
    case EPI_RK4_1:
    case EPI_RK4_2:
    case EPI_RK4_3: {  // rho_n = rho + c*k ; acc = rho + k/6 or acc += k/3 (2/6 on k2+k3)
      const int kind = KIND >= 0 ? KIND : st.kind;
      const double c = kind == EPI_RK4_3 ? 1.0 : 0.5;
      const double w = kind == EPI_RK4_1 ? (1.0 / 6.0) : (2.0 / 6.0);
      double2 a = p.a;
      if constexpr (MIX) {
        // explicit roundings (no contraction), shared with k_rk4_resident
        const float fdt = static_cast<float>(dt);
        const float2 k = make_float2(__fmul_rn(-fdt, Dc.x), __fmul_rn(-fdt, Dc.y));
        static_cast<float2*>(st.Ynext)[g] = make_float2(fmaf(static_cast<float>(c), k.x, p.f.x),
                                                        fmaf(static_cast<float>(c), k.y, p.f.y));
        const double2 kw = to_d(make_float2(__fmul_rn(static_cast<float>(w), k.x), __fmul_rn(static_cast<float>(w), k.y)));
        a.x += kw.x;
        a.y += kw.y;
      } else {
        // explicit FMAs, shared with k_fixed_local
        const double2 k = make_double2(-dt * D.x, -dt * D.y);
        st_bulk<TC>(st.Ynext, g, make_double2(fma(c, k.x, p.b.x), fma(c, k.y, p.b.y)));
        a.x = fma(w, k.x, a.x);
        a.y = fma(w, k.y, a.y);
      }
      __stcs(st.acc + g, a);
      return 0.0;
    }
    case EPI_RK4_4: {  // rho = acc + k4/6
      double2 v;
      if constexpr (MIX) {
        const float fdt = static_cast<float>(dt);
        const double2 k6 = to_d(make_float2(__fmul_rn(1.0f / 6.0f, __fmul_rn(-fdt, Dc.x)),
                                            __fmul_rn(1.0f / 6.0f, __fmul_rn(-fdt, Dc.y))));
        v = make_double2(p.a.x + k6.x, p.a.y + k6.y);
      } else {
        const double2 k = make_double2(-dt * D.x, -dt * D.y);
        v = make_double2(fma(1.0 / 6.0, k.x, p.a.x), fma(1.0 / 6.0, k.y, p.a.y));
      }
      __stcs(st.S[0] + g, v);
      if (st.bulk_separate) st_bulk<TC>(st.Yb[0], g, v);
      return 0.0;
    }
    case EPI_LS: {  // buff = -buff + k (beta=-1) or k (beta=0); rho += B*buff
      if constexpr (MIX) {  // the buffer combines FP32 k's: kept in FP32; the state update is FP64
        // explicit roundings (no contraction), shared with k_ls_resident
        const float fdt = static_cast<float>(dt);
        const float2 b = st.ls_first ? make_float2(__fmul_rn(-fdt, Dc.x), __fmul_rn(-fdt, Dc.y))
                                     : make_float2(fmaf(-fdt, Dc.x, -p.f.x), fmaf(-fdt, Dc.y, -p.f.y));
        __stcs(reinterpret_cast<float2*>(st.acc) + g, b);
        const double2 bd = to_d(b);
        const double2 v = make_double2(fma(st.coef, bd.x, p.b.x), fma(st.coef, bd.y, p.b.y));
        __stcs(st.S[1 - st.ls_in] + g, v);
        if (st.bulk_separate) st_bulk<TC>(st.Yb[1 - st.ls_in], g, v);
      } else {
        const double2 k = make_double2(-dt * D.x, -dt * D.y);
        const double2 b = st.ls_first ? k : make_double2(-p.a.x + k.x, -p.a.y + k.y);
        __stcs(st.acc + g, b);
        const double2 v = make_double2(fma(st.coef, b.x, p.b.x), fma(st.coef, b.y, p.b.y));  // as k_fixed_local
        __stcs(st.S[1 - st.ls_in] + g, v);
        if (st.bulk_separate) st_bulk<TC>(st.Yb[1 - st.ls_in], g, v);
      }
      return 0.0;
    }
    case EPI_DP: {  // store k_s; next stage input rho + sum_j A[s+1][j] k_j
      const int s_ = st.dp_stage;
      if constexpr (MIX) {
        const float fdt = static_cast<float>(dt);
        const float2 k = make_float2(-fdt * Dc.x, -fdt * Dc.y);
        __stcs(static_cast<float2*>(st.K[s_]) + g, k);
        if (s_ < 5) {
          const float c = static_cast<float>(c_dpA[s_ + 1][s_]);
          static_cast<float2*>(st.Ynext)[g] = make_float2(fmaf(c, k.x, p.f.x), fmaf(c, k.y, p.f.y));
        } else {
          float2 hi = p.f, lo = p.g;
          ff_add_prod(hi.x, lo.x, c_dpBh[5], c_dpBl[5], k.x);
          ff_add_prod(hi.y, lo.y, c_dpBh[5], c_dpBl[5], k.y);
          const double2 hd = to_d(hi), ld = to_d(lo);
          const double2 y = make_double2((p.a.x + hd.x) + ld.x, (p.a.y + hd.y) + ld.y);
          __stcs(st.S[1 - cur] + g, y);
          static_cast<float2*>(st.Yb[1 - cur])[g] = to_f(y);
        }
      } else {
        const double2 k = make_double2(-dt * D.x, -dt * D.y);
        st_bulk_cs<TC>(st.K[s_], g, k);
        double2 y = p.a;
        const double c = c_dpA[s_ + 1][s_];
        y.x = fma(c, k.x, y.x);
        y.y = fma(c, k.y, y.y);
        if (s_ < 5)
          st_bulk<TC>(st.Ynext, g, y);
        else
          __stcs(st.S[1 - cur] + g, y);
      }
      return 0.0;
    }
    case EPI_DP7: {  // e = sum_j E_j k_j ; scaled squared error (linalg_engine_cuda.cu:102-146)
      if constexpr (MIX) {  // per-element term in FP32; the sum over elements is FP64
        const float fdt = static_cast<float>(dt);
        const float c = static_cast<float>(c_dpE[6]);
        const float ex = fmaf(c, -fdt * Dc.x, p.f.x), ey = fmaf(c, -fdt * Dc.y, p.f.y);
        const float s = static_cast<float>(st.ctl->atol) +
                        static_cast<float>(st.ctl->rtol) * sqrtf(static_cast<float>(p.m));
        return f2d((ex * ex + ey * ey) / (s * s));
      } else {
        const double2 k7 = make_double2(-dt * D.x, -dt * D.y);
        double2 e = p.a;
        e.x = fma(c_dpE[6], k7.x, e.x);
        e.y = fma(c_dpE[6], k7.y, e.y);
        const double e2 = fma(e.x, e.x, e.y * e.y);
        const double s = fma(st.ctl->rtol, sqrt(p.m), st.ctl->atol);
        return e2 / (s * s);
      }
    }
    default:
      return 0.0;
  }
}

// Both halves at once, for kernels that do not overlap them.
template <typename TC>
__device__ __forceinline__ double epilogue(const Stage& st, size_t g, cx_t<TC> Dc, double dt, int cur) {
  const EpiPre p = epi_pre<TC>(st, g, cur);
  return epi_post<TC>(st, g, Dc, dt, cur, p);
}

// Block-level sum of `v`; result valid in thread 0.
__device__ __forceinline__ double block_sum(double v) {
  __shared__ double warp_part[32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) warp_part[w] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  v = 0.0;
  if (w == 0) {
    v = lane < nw ? warp_part[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// Grid-level finish of the stage-7 error norm: every CTA deposits its partial
// sum; the last CTA to arrive adds them in index order (deterministic) and
// runs the step controller.  No CTA waits on another.
static __device__ void dp7_finish(const Stage& st, double local, long long n_total) {
  const double part = block_sum(local);
  __shared__ bool last;
  if (threadIdx.x == 0) {
    st.partials[blockIdx.x] = part;
    __threadfence();
    const unsigned int ticket = atomicAdd(&st.ctl->arrive, 1u);
    last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  double v = 0.0;
  for (int i = threadIdx.x; i < static_cast<int>(gridDim.x); i += blockDim.x) v += __ldcg(st.partials + i);
  v = block_sum(v);
  if (threadIdx.x == 0) {
    st.ctl->arrive = 0;
    dp_control(st.ctl, v, n_total, st.bulk_separate != 0);
  }
}

template <typename TB>
__device__ __forceinline__ const TB* stage_input(const Stage& st, int cur) {
  if (st.y_sel == 1) return static_cast<const TB*>(st.Yb[cur]);
  if (st.y_sel == 2) return static_cast<const TB*>(st.Yb[1 - cur]);
  return static_cast<const TB*>(st.y_fixed);
}

// Reads the step size and the current buffer index; false if the launch has
// nothing to do (interval finished or failed).
template <int KIND = -1>
__device__ __forceinline__ bool stage_prologue(const Stage& st, double& dt, int& cur) {
  dt = 0.0;
  cur = 0;
  if (st.ctl) {
    if (st.ctl->done || st.ctl->status) return false;
    const int kind = KIND >= 0 ? KIND : st.kind;
    dt = (kind == EPI_DP || kind == EPI_DP7) ? st.ctl->dt : st.ctl->dt_fixed;
    cur = st.ctl->cur;
  }
  return true;
}

// Grid barrier of a cooperative launch (every CTA resident), in the
// arrive/wait pattern of CUTLASS's GenericBarrier, split in two so that a
// CTA can work on its own data between them.  grid_arrive: the CTA syncs,
// one thread adds 1 to a monotonic 64-bit arrival counter with release
// semantics.  grid_wait: that thread spins with acquire loads until the
// counter reaches (gen + 1) * gridDim.x (gen: barriers completed so far),
// then the CTA syncs.  bar[0] is the counter, bar[16] the failure flag (its
// own 128-byte line); both zero at launch.  The spin is bounded; grid_wait
// returns false, CTA-uniformly, if it ran out.
static __device__ __forceinline__ void grid_arrive(unsigned long long* bar, const ResidentArgs& R) {
  __syncthreads();
  // R.skip_arrive_cta: fault injection for tests (that CTA never arrives, so
  // every wait after it runs out); -1 in normal use
  if (threadIdx.x == 0 && static_cast<int>(blockIdx.x) != R.skip_arrive_cta) {
    const unsigned long long one = 1;
    asm volatile("red.release.gpu.global.add.u64 [%0], %1;\n" ::"l"(bar), "l"(one) : "memory");
  }
}
static __device__ bool grid_wait(unsigned long long* bar, unsigned long long& gen, long long spin_limit) {
  __shared__ int s_ok;
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long target = (gen + 1) * gridDim.x;
    for (int it = 0;; ++it) {
      unsigned long long v;
      asm volatile("ld.acquire.gpu.global.u64 %0, [%1];\n" : "=l"(v) : "l"(bar) : "memory");
      if (v >= target) break;
      if (it >= spin_limit) {
        ok = 0;
        atomicOr(bar + 16, 1ull);
        break;
      }
    }
    ++gen;
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

}  // namespace heomgb
