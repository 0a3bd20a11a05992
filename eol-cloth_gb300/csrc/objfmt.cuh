// Text formatting of the OBJ frame files on the device.
//
// The reference writes every number of a frame with C's printf: "%f" (six
// decimals) for coordinates and "%i" for face indices (Cloth.cpp:535-590).
// glibc prints the exact decimal expansion of the binary value rounded to six
// places, ties to even (the round-to-nearest mode), a '-' for any value with
// the sign bit set (also "-0.000000"), and "inf"/"nan" with their signs.
// fmt_f6 restates that rule with integer arithmetic: a double is M * 2^e with
// an integer M < 2^53, so |v| * 10^6 = M * 10^6 * 2^e, a product below 2^73
// shifted by e, rounded on the shifted-out bits.  Values of magnitude 2^63
// and above (integer part beyond 64 bits) are not formatted: the caller
// reports them as an error.
//
// Everything here is __host__ __device__ so the same code is checked against
// the C library's printf on the CPU.
#pragma once

#include <cstdint>
#include <cstring>

namespace eolc {
namespace obj {

// Longest text of one number: sign, 19 integer digits, '.', 6 decimals.
constexpr int kMaxNum = 27;
// Longest line (a face line with three 10-digit indices) plus margin.
constexpr int kMaxLine = 128;

__host__ __device__ inline uint64_t dbits(double v) {
#ifdef __CUDA_ARCH__
  return static_cast<uint64_t>(__double_as_longlong(v));
#else
  uint64_t b;
  memcpy(&b, &v, 8);
  return b;
#endif
}

__host__ __device__ inline int udigits(uint64_t u) {
  int n = 1;
  while (u >= 10) {
    u /= 10;
    ++n;
  }
  return n;
}

// Writes u in decimal at out (if out != nullptr); returns the digit count.
__host__ __device__ inline int put_u64(uint64_t u, char *out) {
  const int n = udigits(u);
  if (out) {
    for (int k = n - 1; k >= 0; --k) {
      out[k] = char('0' + u % 10);
      u /= 10;
    }
  }
  return n;
}

__host__ __device__ inline int put_str(const char *s, char *out) {
  int n = 0;
  while (s[n]) {
    if (out) out[n] = s[n];
    ++n;
  }
  return n;
}

// "%f" of v at out (nullptr: length only).  Returns the length, or -1 when
// |v| >= 2^63.
__host__ __device__ inline int fmt_f6(double v, char *out) {
  const uint64_t b = dbits(v);
  const bool neg = (b >> 63) != 0;
  const int E = int((b >> 52) & 0x7ff);
  const uint64_t frac = b & ((uint64_t(1) << 52) - 1);
  int n = 0;
  if (neg) {
    if (out) out[0] = '-';
    n = 1;
  }
  char *o = out ? out + n : nullptr;
  if (E == 0x7ff) return n + put_str(frac ? "nan" : "inf", o);
  uint64_t M;
  int e;
  if (E == 0) {
    M = frac;
    e = -1074;
  } else {
    M = frac | (uint64_t(1) << 52);
    e = E - 1075;
  }
  if (e >= 11) return -1;  // |v| >= 2^63
  // R = round-half-even(M * 10^6 * 2^e), kept as a 128-bit integer
  unsigned __int128 P = (unsigned __int128)M * 1000000u;
  unsigned __int128 R;
  if (e >= 0) {
    R = P << e;
  } else {
    const int sh = -e;
    if (sh >= 75) {
      R = 0;  // P < 2^73 <= half of 2^sh
    } else {
      R = P >> sh;
      const unsigned __int128 rem = P - (R << sh);
      const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
      if (rem > half || (rem == half && (R & 1))) R += 1;
    }
  }
  if (R >= ((unsigned __int128)1000000u << 63)) return -1;
  // R < 10^6 * 2^63 < 2^83: divide by 10^6 limb by limb (32-bit limbs).  The
  // top limb is below 2^19 < 10^6, so its quotient is 0 and it passes on as
  // the first remainder; each later quotient limb is below 2^32.
  const uint64_t l2 = uint64_t(R >> 64), l1 = uint32_t(R >> 32), l0 = uint32_t(R);
  uint64_t cur = (l2 << 32) | l1;
  const uint64_t q1 = cur / 1000000u;
  cur = ((cur % 1000000u) << 32) | l0;
  const uint64_t q0 = cur / 1000000u;
  const uint32_t fp = uint32_t(cur % 1000000u);
  const uint64_t ip = (q1 << 32) + q0;
  const int ni = put_u64(ip, o);
  if (o) {
    o[ni] = '.';
    uint32_t f = fp;
    for (int k = 6; k >= 1; --k) {
      o[ni + k] = char('0' + f % 10);
      f /= 10;
    }
  }
  return n + ni + 7;
}

// "%i" of a non-negative int.
__host__ __device__ inline int fmt_i(int v, char *out) {
  return put_u64(uint64_t(uint32_t(v)), out);
}

}  // namespace obj
}  // namespace eolc
