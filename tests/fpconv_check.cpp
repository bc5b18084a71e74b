// Checks the integer-assembled FP32 <-> FP64 conversions of the mixed form
// (libheom_gb300/csrc/fpconv.cuh) against the compiler's IEEE conversions:
// every float to double, every float and every midpoint between neighbouring
// floats back to float (ties), and seeded random doubles over the whole
// range.  Prints "ok" or the first mismatch; exit status 0 on success.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <initializer_list>

#include "../libheom_gb300/csrc/fpconv.cuh"

using heomgb::d2f;
using heomgb::f2d;

static uint64_t bits_d(double x) { uint64_t u; std::memcpy(&u, &x, 8); return u; }
static uint32_t bits_f(float x) { uint32_t u; std::memcpy(&u, &x, 4); return u; }
static double from_d(uint64_t u) { double x; std::memcpy(&x, &u, 8); return x; }
static float from_f(uint32_t u) { float x; std::memcpy(&x, &u, 4); return x; }

static bool same_f(float a, float b) { return (std::isnan(a) && std::isnan(b)) || bits_f(a) == bits_f(b); }
static bool same_d(double a, double b) { return (std::isnan(a) && std::isnan(b)) || bits_d(a) == bits_d(b); }

int main(int argc, char** argv) {
  const uint64_t stride = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;  // 1: every float
  for (uint64_t i = 0; i < (1ull << 32); i += stride) {
    const float f = from_f(static_cast<uint32_t>(i));
    const double d = f2d(f);
    if (!same_d(d, static_cast<double>(f))) {
      std::printf("f2d mismatch at %08llx\n", static_cast<unsigned long long>(i));
      return 1;
    }
    if (!same_f(d2f(d), static_cast<float>(d))) {
      std::printf("d2f mismatch (float value) at %08llx\n", static_cast<unsigned long long>(i));
      return 1;
    }
    // midpoint towards the next float of larger magnitude (exact in double): the tie case
    const uint32_t nb = static_cast<uint32_t>(i) + 1u;
    if ((static_cast<uint32_t>(i) & 0x7f800000u) != 0x7f800000u && (nb & 0x7fffffffu) <= 0x7f800000u) {
      const double mid = 0.5 * (d + static_cast<double>(from_f(nb)));
      for (double x : {mid, std::nextafter(mid, 0.0), std::nextafter(mid, 2.0 * mid + 1.0)})
        if (!same_f(d2f(x), static_cast<float>(x))) {
          std::printf("d2f mismatch near midpoint %08llx\n", static_cast<unsigned long long>(i));
          return 1;
        }
    }
  }
  uint64_t s = 0x9e3779b97f4a7c15ull;
  for (int r = 0; r < (1 << 24); ++r) {  // random doubles: full range, then the float range, then subnormal floats
    s ^= s << 13; s ^= s >> 7; s ^= s << 17;
    uint64_t u = s;
    if (r % 3 == 1) u = (u & 0x800fffffffffffffull) | (static_cast<uint64_t>(860 + (s >> 20) % 300) << 52);
    if (r % 3 == 2) u = (u & 0x800fffffffffffffull) | (static_cast<uint64_t>(870 + (s >> 20) % 40) << 52);
    const double x = from_d(u);
    if (!same_f(d2f(x), static_cast<float>(x))) {
      std::printf("d2f mismatch at random %016llx\n", static_cast<unsigned long long>(u));
      return 1;
    }
  }
  std::printf("ok\n");
  return 0;
}
