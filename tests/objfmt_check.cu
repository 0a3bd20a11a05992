// Host check of the device text formatter (eol-cloth_gb300/csrc/objfmt.cuh)
// against the C library's printf: "%f" of doubles and of floats promoted to
// double, and "%i" of face indices.  Runs no device code.
//
// Usage: objfmt_check <random cases>   prints "mismatches N" and exits 1 on any.
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include "../eol-cloth_gb300/csrc/objfmt.cuh"

using namespace eolc::obj;

static long long g_bad = 0, g_cases = 0;

static void check_f(double v) {
  ++g_cases;
  char want[400], got[64];
  int lw = snprintf(want, sizeof(want), "%f", v);
  int lg_only = fmt_f6(v, nullptr);
  if (std::fabs(v) >= 9223372036854775808.0 && std::isfinite(v)) {
    if (lg_only != -1) {
      if (g_bad++ < 20) printf("expected refusal for %.17g, got length %d\n", v, lg_only);
    }
    return;
  }
  int lg = fmt_f6(v, got);
  if (lg < 0 || lg != lg_only || lg != lw || memcmp(want, got, lw) != 0) {
    if (g_bad++ < 20)
      printf("%%f mismatch for %a: printf '%s' formatter '%.*s' (%d, %d)\n", v, want,
             lg < 0 ? 0 : lg, got, lg, lg_only);
  }
}

static void check_i(int v) {
  ++g_cases;
  char want[32], got[32];
  int lw = snprintf(want, sizeof(want), "%i", v);
  int lg = fmt_i(v, got);
  if (lg != lw || memcmp(want, got, lw) != 0) {
    if (g_bad++ < 20) printf("%%i mismatch for %d\n", v);
  }
}

int main(int argc, char **argv) {
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  // exact ties at the sixth decimal (k / 2^7 has 7 binary places = 7 decimal
  // places ending in 5): round half to even
  for (int k = -4096; k <= 4096; ++k) check_f(k / 128.0);
  for (int k = -4096; k <= 4096; ++k) check_f(k / 64.0 + 1e6);
  // every value a few ulps around decimal boundaries d * 1e-6 - 5e-7
  for (int d = -3000; d <= 3000; ++d) {
    double c = d * 1e-6 + 5e-7;
    double lo = c, hi = c;
    for (int u = 0; u < 4; ++u) {
      lo = nextafter(lo, -INFINITY);
      hi = nextafter(hi, INFINITY);
      check_f(lo);
      check_f(hi);
    }
    check_f(c);
  }
  // signed zeros, tiny values, subnormals, infinities, NaNs, range limits
  const double special[] = {0.0, -0.0, 5e-7, -5e-7, 4.9999999999999e-7, 5.0000000000001e-7,
                            DBL_MIN, -DBL_MIN, 4.9e-324, -4.9e-324, INFINITY, -INFINITY,
                            NAN, -NAN, 9223372036854775807.0, 9223372036854774784.0,
                            -9223372036854774784.0, 4503599627370496.5, 999999.9999995,
                            0.9999995, 0.99999949999999994, 1e15 + 0.3, FLT_MAX, -FLT_MAX,
                            1e300, 9.5, 0.5, 1.5, 2.5};
  for (double v : special) check_f(v);
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> unit(-1.0, 1.0);
  std::uniform_int_distribution<int> expo(-40, 66);
  for (long long k = 0; k < n; ++k) {
    // doubles over many binades, and the float-rounded values the files hold
    double v = std::ldexp(unit(rng), expo(rng));
    check_f(v);
    check_f(double(float(v)));
    uint64_t bits = rng();
    double r;
    memcpy(&r, &bits, 8);
    check_f(r);  // arbitrary bit patterns (mostly refused or tiny)
  }
  const int ints[] = {0, 1, 9, 10, 99, 100, 12345, 999999999, 1000000000, 2147483647};
  for (int v : ints) check_i(v);
  std::uniform_int_distribution<int> iu(0, 2147483647);
  for (int k = 0; k < 100000; ++k) check_i(iu(rng));
  printf("cases %lld mismatches %lld\n", g_cases, g_bad);
  return g_bad ? 1 : 0;
}
