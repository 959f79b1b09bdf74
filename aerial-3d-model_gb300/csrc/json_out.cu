// Number text of the sparse stage's cameras.json, host code: serde_json
// writes an f64 in the shortest form that reads back to the same value
// (mod.rs:30, `serde_json::to_vec`), laid out as
//   integral values below 1e16          1234.0
//   1e-5 <= |x| < 1e16                  12.34, 0.0001234
//   otherwise                           1e30, 1.234e-7 (no '+', no padding)
// with -0.0 as "-0.0" and non-finite values as null.  The shortest digits come
// from std::to_chars; the layout above is applied to them here.
#include <charconv>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "ba_gb300.h"
#include "context.cuh"

namespace ba {
namespace {

// Writes x at p, returns the number of characters (at most 25).
int format_f64(double x, char* p) {
  if (!std::isfinite(x)) {
    std::memcpy(p, "null", 4);
    return 4;
  }
  int n = 0;
  if (std::signbit(x)) p[n++] = '-', x = -x;
  if (x == 0.0) {
    std::memcpy(p + n, "0.0", 3);
    return n + 3;
  }
  char sci[40];
  const auto r = std::to_chars(sci, sci + sizeof sci, x, std::chars_format::scientific);
  // sci = d[.ddd]e(+|-)XX
  char dig[24];
  int len = 0, i = 0;
  dig[len++] = sci[i++];
  if (sci[i] == '.')
    for (++i; sci[i] != 'e'; ++i) dig[len++] = sci[i];
  int e = 0;
  {
    const char* q = sci + i + 1;
    const bool neg = *q == '-';
    if (*q == '+' || *q == '-') ++q;
    for (; q < r.ptr; ++q) e = 10 * e + (*q - '0');
    if (neg) e = -e;
  }
  while (len > 1 && dig[len - 1] == '0') --len;
  const int kk = e + 1;     // 10^(kk-1) <= x < 10^kk
  const int k = kk - len;   // x = digits * 10^k
  if (k >= 0 && kk <= 16) {
    std::memcpy(p + n, dig, len), n += len;
    for (int j = 0; j < k; ++j) p[n++] = '0';
    p[n++] = '.', p[n++] = '0';
  } else if (kk > 0 && kk <= 16) {
    std::memcpy(p + n, dig, kk), n += kk;
    p[n++] = '.';
    std::memcpy(p + n, dig + kk, len - kk), n += len - kk;
  } else if (kk > -5 && kk <= 0) {
    p[n++] = '0', p[n++] = '.';
    for (int j = 0; j < -kk; ++j) p[n++] = '0';
    std::memcpy(p + n, dig, len), n += len;
  } else {
    p[n++] = dig[0];
    if (len > 1) {
      p[n++] = '.';
      std::memcpy(p + n, dig + 1, len - 1), n += len - 1;
    }
    p[n++] = 'e';
    int x10 = kk - 1;
    if (x10 < 0) p[n++] = '-', x10 = -x10;
    char t[8];
    int m = 0;
    do t[m++] = (char)('0' + x10 % 10), x10 /= 10;
    while (x10);
    while (m) p[n++] = t[--m];
  }
  return n;
}

int format_u64(uint64_t v, char* p) {
  char t[24];
  int m = 0, n = 0;
  do t[m++] = (char)('0' + v % 10), v /= 10;
  while (v);
  while (m) p[n++] = t[--m];
  return n;
}

template <typename T, typename F>
void rows_json(const T* v, int64_t n, int32_t group, char* out, int64_t cap, int64_t* len,
               int per_value, F fmt) {
  if (n < 0 || group < 0 || (group > 0 && n % group)) throw BadInput("bad array shape");
  if (n > 0 && !v) throw BadInput("null array");
  if (!out || !len) throw BadInput("null output");
  const int64_t need = n * (per_value + 1) + 2 * (group > 0 ? n / group : 0) + 2 + 1;
  if (cap < need) throw BadInput("output buffer too small");
  int64_t o = 0;
  out[o++] = '[';
  for (int64_t i = 0; i < n; ++i) {
    if (i) out[o++] = ',';
    if (group > 0 && i % group == 0) out[o++] = '[';
    o += fmt(v[i], out + o);
    if (group > 0 && i % group == group - 1) out[o++] = ']';
  }
  out[o++] = ']';
  out[o] = 0;
  *len = o;
}

}  // namespace
}  // namespace ba

using namespace ba;

extern "C" ba_status ba_json_f64(const double* v, int64_t n, int32_t group, char* out,
                                 int64_t cap, int64_t* len) {
  return guarded([&] { rows_json(v, n, group, out, cap, len, 25, format_f64); });
}

extern "C" ba_status ba_json_u8(const uint8_t* v, int64_t n, int32_t group, char* out,
                                int64_t cap, int64_t* len) {
  return guarded([&] {
    rows_json(v, n, group, out, cap, len, 3, [](uint8_t x, char* p) { return format_u64(x, p); });
  });
}

extern "C" ba_status ba_json_u32(const uint32_t* v, int64_t n, int32_t group, char* out,
                                 int64_t cap, int64_t* len) {
  return guarded([&] {
    rows_json(v, n, group, out, cap, len, 10, [](uint32_t x, char* p) { return format_u64(x, p); });
  });
}
