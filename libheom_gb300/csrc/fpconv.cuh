// Exact FP32 <-> FP64 conversions assembled from the IEEE-754 encodings with
// integer operations.  On this part the FP64 pipe executes about two
// operations per clock per SM, and the conversion instructions (float ->
// double, double -> float, int -> double) issue there too; the mixed form
// converts every element in every stage, so these versions keep the FP64
// pipe for the FP64 arithmetic itself.  Both give the bits of the IEEE
// conversions (float -> double is exact; double -> float rounds to nearest,
// ties to even, with overflow to infinity and gradual underflow); NaNs stay
// NaNs (quiet, payload truncated).  Host-callable so that the same code is
// checked exhaustively on the CPU against the compiler's own conversions.
#pragma once

#include <cstdint>
#include <cstring>

#if defined(__CUDACC__)
#define HEOMGB_HD __host__ __device__ __forceinline__
#else
#define HEOMGB_HD inline
#endif

namespace heomgb {

HEOMGB_HD uint32_t fc_f2u(float x) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(x);
#else
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return u;
#endif
}
HEOMGB_HD float fc_u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float x;
  std::memcpy(&x, &u, 4);
  return x;
#endif
}
HEOMGB_HD uint64_t fc_d2u(double x) {
#if defined(__CUDA_ARCH__)
  return static_cast<uint64_t>(__double_as_longlong(x));
#else
  uint64_t u;
  std::memcpy(&u, &x, 8);
  return u;
#endif
}
HEOMGB_HD double fc_u2d(uint64_t u) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double(static_cast<long long>(u));
#else
  double x;
  std::memcpy(&x, &u, 8);
  return x;
#endif
}
// index of the most significant set bit of v != 0
HEOMGB_HD int fc_msb(uint32_t v) {
#if defined(__CUDA_ARCH__)
  return 31 - __clz(static_cast<int>(v));
#else
  return 31 - __builtin_clz(v);
#endif
}

#if defined(__CUDA_ARCH__)
#define HEOMGB_COLD static __device__ __noinline__
#else
#define HEOMGB_COLD static inline
#endif

// float -> double (exact).  The common case (a normal float) is a few integer
// operations; zeros, subnormals, infinities and NaNs take a separate call so
// that the compiler does not predicate their paths into every conversion.
HEOMGB_COLD uint64_t f2d_rare(uint32_t u) {
  const uint64_t sign = static_cast<uint64_t>(u >> 31) << 63;
  const uint32_t ex = (u >> 23) & 0xffu, man = u & 0x7fffffu;
  if (ex == 0xffu) return sign | (0x7ffull << 52) | (static_cast<uint64_t>(man) << 29);  // infinity or NaN
  if (man == 0) return sign;                                                           // signed zero
  const int p = fc_msb(man);  // subnormal: man * 2^-149 with its leading bit at position p
  return sign | (static_cast<uint64_t>(p + 874) << 52) | ((static_cast<uint64_t>(man) << (52 - p)) & ((1ull << 52) - 1));
}
HEOMGB_HD double f2d(float x) {
  const uint32_t u = fc_f2u(x);
  const uint32_t ex = (u >> 23) & 0xffu;
  if (ex - 1u < 0xfeu)  // normal: rebias the exponent (1023 - 127), widen the fraction
    return fc_u2d((static_cast<uint64_t>(u >> 31) << 63) | (static_cast<uint64_t>(ex + 896u) << 52) |
                  (static_cast<uint64_t>(u & 0x7fffffu) << 29));
  return fc_u2d(f2d_rare(u));
}

// double -> float, round to nearest even.  The common case (a result in the
// normal float range) drops 29 fraction bits with one rounding increment (a
// carry may reach the exponent, up to infinity); the rest takes a separate call.
HEOMGB_COLD uint32_t d2f_rare(uint64_t u) {
  const uint32_t sign = static_cast<uint32_t>(u >> 63) << 31;
  const int ex = static_cast<int>((u >> 52) & 0x7ffu);
  const uint64_t man = u & ((1ull << 52) - 1);
  if (ex == 0x7ff)  // infinity, or a quiet NaN
    return sign | 0x7f800000u | (man ? (0x400000u | static_cast<uint32_t>(man >> 29)) : 0u);
  if (ex - 896 >= 255) return sign | 0x7f800000u;  // overflow
  // subnormal or zero result: q = round(M / 2^s), M the 53-bit significand
  const int s = 926 - ex;  // >= 30
  if (s > 54 || ex == 0) return sign;  // below half the smallest subnormal (FP64 subnormals too)
  const uint64_t M = man | (1ull << 52);
  uint32_t q = static_cast<uint32_t>(M >> s);
  const uint64_t rem = M & ((1ull << s) - 1), half = 1ull << (s - 1);
  if (rem > half || (rem == half && (q & 1u))) q += 1u;  // may become the smallest normal: same encoding
  return sign | q;
}
HEOMGB_HD float d2f(double x) {
  const uint64_t u = fc_d2u(x);
  const uint32_t hi = static_cast<uint32_t>(u >> 32);
  const uint32_t e = ((hi >> 20) & 0x7ffu) - 897u;  // biased float exponent - 1, unsigned
  if (e < 254u) {  // the float exponent is 1..254
    // sign | exponent | the top 23 fraction bits, then round on the 29 dropped bits
    uint32_t bits = (hi & 0x80000000u) | ((e + 1u) << 23) | static_cast<uint32_t>((u >> 29) & 0x7fffffu);
    const uint32_t rem = static_cast<uint32_t>(u) & 0x1fffffffu;
    bits += (rem > 0x10000000u || (rem == 0x10000000u && (bits & 1u))) ? 1u : 0u;
    return fc_u2f(bits);
  }
  return fc_u2f(d2f_rare(u));
}

}  // namespace heomgb
