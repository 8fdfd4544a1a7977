// Host check of the integer-pipe double helpers of device_common.cuh (dkey, ifloor_d, modf_d,
// itrunc_d, double_of_int, dmin_k, dmax_k, is_nan_bits, sin_cos_series_short) against the C library on many values: powers of two and their neighbours, integers
// and near-integers of both signs, signed zeros and random values over 40 binades.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "../../mithra_gb300/csrc/device_common.cuh"

using namespace mithra;

int main() {
  // NaNs and infinities only for is_nan_bits (the other helpers are not defined on them)
  const double special[] = {std::nan(""), -std::nan(""), (double)INFINITY, -(double)INFINITY, 1e308, -1e308};
  for (double x : special)
    if (is_nan_bits(x) != std::isnan(x)) { printf("is_nan_bits(%g)\n", x); return 1; }
  std::vector<double> v = {0.0, -0.0, 1.0, -1.0, 0.5, -0.5, 1e-300, -1e-300, 4.9e-324, -4.9e-324,
                           2147483647.0, -2147483647.0, 2147483646.5, -2147483646.5};
  for (int e = -60; e <= 30; e++) {
    const double p = std::ldexp(1.0, e);
    for (double x : {p, std::nextafter(p, 0.0), std::nextafter(p, 1e300)}) {
      v.push_back(x);
      v.push_back(-x);
    }
  }
  for (int i = -3000; i <= 3000; i++) {
    v.push_back((double)i);
    v.push_back(std::nextafter((double)i, 1e300));
    v.push_back(std::nextafter((double)i, -1e300));
    v.push_back(i + 0.25);
  }
  std::mt19937_64 rng(12345);
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-40, 30);
  for (int i = 0; i < 200000; i++) v.push_back(std::ldexp(u(rng), ex(rng)));
  long long bad = 0, checks = 0;
  for (size_t a = 0; a < v.size(); a++) {
    const double t = v[a];
    if (std::fabs(t) < 2147483647.0) {
      checks++;
      if (ifloor_d(t) != (int)std::floor(t)) { if (bad++ < 10) printf("ifloor_d(%.17g) = %d\n", t, ifloor_d(t)); }
      double ip1, ip2;
      const double f1 = modf_d(t, &ip1), f2 = std::modf(t, &ip2);
      if (!(f1 == f2 && ip1 == ip2)) { if (bad++ < 10) printf("modf_d(%.17g) = %.17g, %.17g\n", t, f1, ip1); }
      if (itrunc_d(ip1) != (int)std::trunc(t)) { if (bad++ < 10) printf("itrunc_d(%.17g) = %d\n", ip1, itrunc_d(ip1)); }
    }
    if (std::fabs(t) < 2147483647.0) {
      const int n = (int)std::trunc(t);
      checks++;
      if (double_of_int(n) != (double)n) { if (bad++ < 10) printf("double_of_int(%d) = %.17g\n", n, double_of_int(n)); }
    }
    checks++;
    if (is_nan_bits(t) != std::isnan(t)) { if (bad++ < 10) printf("is_nan_bits(%.17g)\n", t); }
    const double s = v[(a * 7919 + 13) % v.size()];
    checks++;
    if (!(dmin_k(t, s) == std::fmin(t, s) && dmax_k(t, s) == std::fmax(t, s))) {
      if (bad++ < 10) printf("dmin_k/dmax_k %.17g %.17g\n", t, s);
    }
    if ((dkey(t) < dkey(s)) != (t < s) || (dkey(t) == dkey(s)) != (t == s)) {
      if (bad++ < 10) printf("dkey order %.17g vs %.17g\n", t, s);
    }
  }
  // sin_cos_series_short on [-1/4, 1/4] against the C library: within 4e-16 absolute
  double worst = 0.0;
  for (int i = -200000; i <= 200000; i++) {
    const double d = 0.25 * i / 200000.0;
    double s, c;
    sin_cos_series_short(d, &s, &c);
    worst = std::fmax(worst, std::fmax(std::fabs(s - std::sin(d)), std::fabs(c - std::cos(d))));
  }
  checks++;
  if (!(worst <= 4e-16)) { bad++; printf("sin_cos_series_short worst error %.3e\n", worst); }
  printf("%s %lld checks, %lld mismatches (sin_cos_series_short worst %.2e)\n", bad ? "FAIL" : "ok", checks, bad, worst);
  return bad ? 1 : 0;
}
