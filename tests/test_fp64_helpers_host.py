"""The FP64 step's exact helpers in step_fp64.cu, on the CPU. Their source
text is taken from the CUDA file as it stands and compiled for the host,
the intrinsics it uses mapped to host equivalents (the host's fma is
correctly rounded, as the GPU's is), then compared bit for bit (NaNs as
NaNs) on random and edge-case operands:
- the integer-pipe additions (sadd, ssub) with IEEE addition;
- the division by a row metric with its correctly rounded reciprocal
  (div_rcp) with IEEE division, and the power-of-two scalings (mul_pow2)
  with IEEE multiplication;
- the limiters on integer images (limiter_fast) with the literal limiters,
  up to the sign of a zero;
- the range test behind the checks (range_bad) with the reference's check
  outcome for one value.
The GPU self-checks (tests/test_division.py) run the first two on the device."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "sw2_gb300", "csrc", "step_fp64.cu")


def function_text(src, signature):
    start = src.index(signature)
    depth, i = 0, src.index("{", start)
    while True:
        if src[i] == "{":
            depth += 1
        elif src[i] == "}":
            depth -= 1
            if depth == 0:
                return src[start:i + 1]
        i += 1


HARNESS = r"""
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
static inline long long dbits(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
static inline double __longlong_as_double(long long b) { double r; std::memcpy(&r, &b, 8); return r; }
static inline int __clzll(long long x) { return __builtin_clzll((unsigned long long)x); }
static double add_fp64(double a, double b) { return a + b; }
%s
%s
static uint64_t st = 0x9E3779B97F4A7C15ULL;
static uint64_t next() {  // SplitMix64
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double mk(uint64_t r, int e, bool neg) {
  return __longlong_as_double((long long)(((uint64_t)e << 52) | (r & 0xFFFFFFFFFFFFFULL) | (neg ? 1ULL << 63 : 0)));
}
static bool isnan_bits(double x) { return (dbits(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
static bool same(double want, double got) {
  if (isnan_bits(want)) return isnan_bits(got);
  return dbits(want) == dbits(got);
}
int main(int argc, char** argv) {
  long long n = atoll(argv[1]), bad = 0;
  for (long long t = 0; t < n; t++) {
    const uint64_t r1 = next(), r2 = next(), r3 = next();
    double a, b;
    switch (r3 %% 8) {
      case 0: a = mk(r1, 1 + (r3 >> 8) %% 2046, r2 & 1); b = mk(r2, 1 + (r3 >> 20) %% 2046, r2 & 2); break;
      case 1: case 2: {  // exponents within 64: alignment, carries, cancellation
        const int e = 70 + (r3 >> 8) %% 1900;
        a = mk(r1, e, r2 & 1); b = mk(r2, e - (int)((r3 >> 20) %% 64), r2 & 2); break;
      }
      case 3:  // b = -a give or take a few ulps
        a = mk(r1, 3 + (r3 >> 8) %% 2040, r2 & 1);
        b = __longlong_as_double((dbits(a) ^ (long long)0x8000000000000000ULL) + (long long)((r2 >> 8) %% 9) - 4);
        break;
      case 4: {  // ties: an odd multiple of half an ulp of a, or next to one
        const int e = 60 + (r3 >> 8) %% 1900;
        a = mk(r1, e, r2 & 1);
        b = (double)(2 * ((r2 >> 8) %% 16) + 1) * mk(0, e - 53, false);
        if (r2 & 4) b = __longlong_as_double(dbits(b) + (long long)((r2 >> 20) %% 3) - 1);
        if (r2 & 2) b = -b;
        break;
      }
      case 5: a = mk(r1, 2046 - (r3 >> 8) %% 3, r2 & 1); b = mk(r2, 2046 - (r3 >> 20) %% 60, r2 & 2); break;
      case 6: a = mk(r1, (r3 >> 8) %% 4, r2 & 1); b = mk(r2, (r3 >> 20) %% 60, r2 & 2); break;
      default: {  // zeros, inf, NaN, against anything
        const double sp[6] = {0.0, -0.0, __longlong_as_double(0x7ff0000000000000LL),
                              __longlong_as_double((long long)0xfff0000000000000ULL),
                              __longlong_as_double(0x7ff8000000000000LL), 1.0};
        a = sp[(r3 >> 8) %% 6];
        b = (r2 & 1) ? sp[(r3 >> 20) %% 6] : mk(r2, 1 + (r3 >> 24) %% 2046, r2 & 2);
        if (r2 & 4) { const double t2 = a; a = b; b = t2; }
      }
    }
    if (!same(a + b, sadd(a, b))) bad++;
    if (!same(a - b, ssub(a, b))) bad++;
  }
  printf("%%lld\n", bad);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_pipe_addition_source_matches_ieee_on_the_host(tmp_path):
    src = open(SRC).read()
    sadd = function_text(src, "__device__ __forceinline__ double sadd(double a, double b) {")
    ssub = function_text(src, "__device__ __forceinline__ double ssub(double a, double b) {")
    sadd, ssub = (re.sub(r"__device__ __forceinline__", "static inline", f) for f in (sadd, ssub))
    c = tmp_path / "soft_add.cpp"
    c.write_text(HARNESS % (sadd, ssub))
    exe = tmp_path / "soft_add"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-o", str(exe), str(c)], check=True)
    out = subprocess.run([str(exe), str(40_000_000)], check=True, capture_output=True, text=True).stdout
    assert int(out.strip()) == 0


DIV_HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
static inline long long dbits(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
static inline double __longlong_as_double(long long b) { double r; std::memcpy(&r, &b, 8); return r; }
static inline int dexp(double x) { return (int)(((unsigned long long)dbits(x) >> 52) & 0x7ffULL); }
static inline double __dmul_rn(double a, double b) { return a * b; }
static inline double __fma_rn(double a, double b, double c) { return std::fma(a, b, c); }
static double mul_pow2_fp64(double x, double p) { return x * p; }
%s
%s
static uint64_t st = 0x243F6A8885A308D3ULL;
static uint64_t next() {
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double mk(uint64_t r, int e, bool neg) {
  return __longlong_as_double((long long)(((uint64_t)e << 52) | (r & 0xFFFFFFFFFFFFFULL) | (neg ? 1ULL << 63 : 0)));
}
static bool same(double want, double got) {
  const bool n1 = (dbits(want) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
  const bool n2 = (dbits(got) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL;
  return n1 ? n2 : dbits(want) == dbits(got);
}
int main(int argc, char** argv) {
  long long n = atoll(argv[1]), bad_div = 0, bad_pow = 0;
  for (long long t = 0; t < n; t++) {
    const uint64_t r1 = next(), r2 = next(), r3 = next();
    // divisors: positive normal numbers over the range of metric factors and
    // beyond, including all-ones significands and powers of two
    double b = mk(r2, 1023 - 40 + (int)((r3 >> 40) %% 90), false);
    if ((r3 & 15) == 0) b = mk(~0ULL, 1023 - 40 + (int)((r3 >> 40) %% 90), false);
    if ((r3 & 15) == 1) b = mk(0, 1023 - 40 + (int)((r3 >> 40) %% 90), false);
    const double y = 1.0 / b;
    double a;
    if (r3 & 16) {  // random numerators, every exponent, both signs, zeros
      a = mk(r1, (int)((r3 >> 8) %% 2047), r3 & 32);
    } else {  // a = b * (q + half an ulp of q, give or take a little): quotient near a midpoint
      const int e = 523 + (int)((r3 >> 8) %% 500);
      const double q = mk(r1, e, false);
      const double h = mk(0, e - 53, false) * (double)(((r3 >> 20) & 7) + 1) * 0.5;
      a = b * (q + h);
      if (r3 & 64) a = __longlong_as_double(dbits(a) + (long long)((r3 >> 24) %% 5) - 2);
    }
    if (!same(a / b, div_rcp(a, b, y))) bad_div++;
    // power-of-two scalings of anything, the exponent field's edges included
    const double x = mk(r1, (r3 & 128) ? (int)((r3 >> 8) %% 2048) : ((r3 & 256) ? (int)((r3 >> 8) %% 4) : 2043 + (int)((r3 >> 8) %% 5)), r3 & 512);
    if (!same(x * 0.5, mul_pow2(x, -1, 0.5))) bad_pow++;
    if (!same(x * 0.25, mul_pow2(x, -2, 0.25))) bad_pow++;
    if (!same(x * 2.0, mul_pow2(x, 1, 2.0))) bad_pow++;
  }
  // every divisor within 512 ulps below 2 or just above 1 against every
  // numerator within 512 ulps below +-2: the pairs where RN(a*y) can stray
  // more than one ulp from a/b
  for (int j = 0; j < 1024; j++) {
    const double b = j < 512 ? __longlong_as_double(0x3FFFFFFFFFFFFFFFLL - j)
                             : __longlong_as_double(0x3FF0000000000000LL + (j - 512));
    const double y = 1.0 / b;
    for (int k = 0; k < 1024; k++) {
      const double a = __longlong_as_double((long long)((0x3FFFFFFFFFFFFFFFULL - (uint64_t)(k & 511)) |
                                                        ((uint64_t)(k >> 9) << 63)));
      if (!same(a / b, div_rcp(a, b, y))) bad_div++;
    }
  }
  printf("%%lld %%lld\n", bad_div, bad_pow);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_metric_division_and_power_of_two_scaling_sources_match_ieee_on_the_host(tmp_path):
    src = open(SRC).read()
    div = function_text(src, "__device__ __forceinline__ double div_rcp(double a, double b, double y) {")
    pw = function_text(src, "__device__ __forceinline__ double mul_pow2(double x, int k, double p) {")
    div, pw = (re.sub(r"__device__ __forceinline__", "static inline", f) for f in (div, pw))
    c = tmp_path / "div.cpp"
    c.write_text(DIV_HARNESS % (pw, div))
    exe = tmp_path / "div"
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-o", str(exe), str(c)], check=True)
    out = subprocess.run([str(exe), str(4_000_000)], check=True, capture_output=True, text=True).stdout
    assert out.split() == ["0", "0"]


LIMITER_HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
constexpr int kVanLeerSafe = 10;
static inline long long dbits(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
static inline double __longlong_as_double(long long b) { double r; std::memcpy(&r, &b, 8); return r; }
static double mul_pow2_fp64(double x, double p) { return x * p; }
%s
#define HALF(x) mul_pow2((x), -1, 0.5)
#define QUARTER(x) mul_pow2((x), -2, 0.25)
#define TWICE(x) mul_pow2((x), 1, 2.0)
%s
%s
%s
%s
%s
static bool ok(double want, double got) {  // equal, or both zeros
  if (dbits(want) == dbits(got)) return true;
  return want == 0.0 && got == 0.0;
}
static uint64_t st = 0x13198A2E03707344ULL;
static uint64_t next() {
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
template <int SCH> long long check(long long n) {
  long long bad = 0;
  const double fixed[] = {0.0, -0.0, 1.0, -1.0, 0.5, 2.0, 1.0 / 3.0, 3.0, 0.25, 0.75, 4.0, 1e-300, -1e-300,
                          1e300, -1e300, 0x1p498, -0x1p498, 0x1p-1022, -0x1p-1022, 5e-324};
  for (double r : fixed) {
    if (!ok(limiter<SCH>(r), limiter_fast<SCH>(r))) bad++;
    for (int k = -3; k <= 3; k++) {
      const double s = __longlong_as_double(dbits(r) + k);
      if (std::isfinite(s) && !ok(limiter<SCH>(s), limiter_fast<SCH>(s))) bad++;
    }
  }
  for (long long t = 0; t < n; t++) {
    const uint64_t a = next(), b = next();
    // ratios of limiter interest (|r| around 1) most of the time, any finite value otherwise
    const int e = (b & 3) ? 1023 - 8 + (int)((b >> 8) %% 16) : (int)((b >> 8) %% 2047);
    const double r = __longlong_as_double((long long)(((uint64_t)e << 52) | (a & 0xFFFFFFFFFFFFFULL) | ((b >> 40) & 1 ? 1ULL << 63 : 0)));
    if (!ok(limiter<SCH>(r), limiter_fast<SCH>(r))) bad++;
  }
  return bad;
}
int main(int argc, char** argv) {
  const long long n = atoll(argv[1]);
  printf("%%lld %%lld %%lld %%lld %%lld %%lld\n", check<0>(n), check<1>(n), check<2>(n), check<4>(n), check<7>(n),
         check<kVanLeerSafe>(n));
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fast_limiters_source_matches_the_literal_limiters_on_the_host(tmp_path):
    """limiter_fast (integer-image comparisons, exponent-field scalings) gives
    the literal limiter's value for every finite ratio, up to the sign of a
    zero (the fast bodies recompute cells whose sum is zero literally)."""
    src = open(SRC).read()
    pw = function_text(src, "__device__ __forceinline__ double mul_pow2(double x, int k, double p) {")
    key = function_text(src, "__device__ __forceinline__ long long key(double x) {")
    one_liners = [ln for ln in src.splitlines()
                  if ln.startswith("__device__ __forceinline__ double mn(") or
                  ln.startswith("__device__ __forceinline__ double mx(")]
    assert len(one_liners) == 2
    one_liners.append(function_text(src, "__device__ __forceinline__ double zdiv(double a, double b) {"))
    lim = "template <int SCH>\n" + function_text(src, "__device__ __forceinline__ double limiter(double r) {")
    fast = "template <int SCH>\n" + function_text(src, "__device__ __forceinline__ double limiter_fast(double r) {")
    parts = [pw, key, "\n".join(one_liners), lim, fast]
    parts = [re.sub(r"__device__ __forceinline__", "static inline", f) for f in parts]
    c = tmp_path / "lim.cpp"
    c.write_text(LIMITER_HARNESS % (parts[0], parts[1], parts[2], parts[3], parts[4], ""))
    exe = tmp_path / "lim"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-o", str(exe), str(c)],
                   check=True)
    out = subprocess.run([str(exe), str(2_000_000)], check=True, capture_output=True, text=True).stdout
    assert out.split() == ["0"] * 6


RANGE_HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
static inline long long dbits(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
static inline double from(uint64_t b) { double r; std::memcpy(&r, &b, 8); return r; }
%s
int main() {
  long long bad = 0, n = 0;
  const double lim = 1e10;
  const double edge[] = {lim, std::nextafter(lim, 0.0), std::nextafter(lim, 1e300), -lim, 0.0, -0.0, 1.0,
                         INFINITY, -INFINITY, NAN, -NAN, 1e300, 5e-324};
  auto test = [&](double x) {
    for (int first = 0; first < 2; first++) {
      // the reference: the first value seeds min and max (a non-finite one fails the check);
      // later NaNs never win a comparison; the step aborts on min < -1e10 or max > 1e10
      const bool want = first ? (!std::isfinite(x) || std::fabs(x) > lim) : (std::fabs(x) > lim);
      if (range_bad(x, first) != want) bad++;
      n++;
    }
  };
  for (double x : edge) test(x);
  uint64_t s = 0x452821E638D01377ULL;
  for (long long t = 0; t < 20000000; t++) {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    const uint64_t b = s ^ (s >> 29);
    test(from((b & 1) ? b : ((b & 0x800FFFFFFFFFFFFFULL) | ((uint64_t)(1023 + 30 + (int)((b >> 52) %% 8)) << 52))));
  }
  printf("%%lld %%lld\n", bad, n);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_range_check_source_matches_the_reference_predicate_on_the_host(tmp_path):
    """range_bad, the bit test behind the range checks, against the
    reference's check_stats_scaf outcome for one value (first or not)."""
    src = open(SRC).read()
    rb = function_text(src, "__device__ __forceinline__ bool range_bad(double x, bool first) {")
    rb = re.sub(r"__device__ __forceinline__", "static inline", rb)
    c = tmp_path / "range.cpp"
    c.write_text(RANGE_HARNESS % rb)
    exe = tmp_path / "range"
    subprocess.run(["g++", "-O2", "-fno-fast-math", "-o", str(exe), str(c)], check=True)
    bad, n = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()
    assert int(bad) == 0 and int(n) > 0


ZDIV_HARNESS = r"""
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
static inline long long dbits(double x) { long long r; std::memcpy(&r, &x, 8); return r; }
static inline double __longlong_as_double(long long b) { double r; std::memcpy(&r, &b, 8); return r; }
%s
static uint64_t st = 0x2545F4914F6CDD1DULL;
static uint64_t next() {  // SplitMix64
  uint64_t z = (st += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static bool isnan_bits(double x) { return (dbits(x) & 0x7fffffffffffffffLL) > 0x7ff0000000000000LL; }
static bool same(double want, double got) {
  if (isnan_bits(want)) return isnan_bits(got);
  return dbits(want) == dbits(got);
}
int main(int argc, char** argv) {
  const double edge[] = {0.0, -0.0, 1.0, -1.0, 5e-324, -5e-324, 2.2250738585072014e-308, 1.7976931348623157e308,
                         INFINITY, -INFINITY, NAN, -NAN, 3.0, -7.5e-300};
  long long bad = 0;
  const int ne = sizeof(edge) / sizeof(edge[0]);
  for (int i = 0; i < ne; i++)
    for (int k = 0; k < ne; k++) bad += !same(edge[i] / edge[k], zdiv(edge[i], edge[k]));
  const long long n = atoll(argv[1]);
  for (long long t = 0; t < n; t++) {
    const uint64_t r1 = next(), r2 = next();
    double a = __longlong_as_double((long long)r1), b = __longlong_as_double((long long)r2);
    if (r1 & 1) a = (r1 & 2) ? -0.0 : 0.0;  // half the numerators zero
    bad += !same(a / b, zdiv(a, b));
  }
  printf("%%lld\n", bad);
  return 0;
}
"""


def test_zero_numerator_division_source_matches_ieee_on_the_host(tmp_path):
    """zdiv (the literal cells' division, a zero numerator answered from the
    bits) equals IEEE division bit for bit (NaNs as NaNs) on every pair of
    edge values (zeros of both signs, subnormals, the extremes, infinities,
    NaNs) and on random bit patterns, half of them with zero numerators."""
    src = open(SRC).read()
    z = function_text(src, "__device__ __forceinline__ double zdiv(double a, double b) {")
    z = re.sub(r"__device__ __forceinline__", "static inline", z)
    c = tmp_path / "zdiv.cpp"
    c.write_text(ZDIV_HARNESS % z)
    exe = tmp_path / "zdiv"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-o", str(exe), str(c)],
                   check=True)
    out = subprocess.run([str(exe), str(2_000_000)], check=True, capture_output=True, text=True).stdout
    assert out.split() == ["0"]
