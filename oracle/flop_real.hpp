// flop_real.hpp -- an FP64 scalar that counts the arithmetic done with it.
//
// TEST INFRASTRUCTURE ONLY.  oracle_count.cpp compiles the oracle's
// restatement of the reference (rxn_oracle.hpp) with every double replaced by
// Real, so that one run of RStep reports the floating-point work the
// reference algorithm does: add, subtract, multiply, divide and square root
// count one flop each (fused multiply-add two), exp / log / pow are counted
// separately as transcendental calls, comparisons, fabs and sign changes are
// free.  The values are computed in plain double, so the counted run gives
// the same results as the oracle.
#pragma once
#include <cmath>

namespace flopcount {
struct Counters {
  long long flops = 0;
  long long transcendentals = 0;
};
inline Counters& counters() {
  static thread_local Counters c;
  return c;
}
}  // namespace flopcount

struct Real {
  double v;
  constexpr Real() : v(0.0) {}
  constexpr Real(double x) : v(x) {}  // NOLINT: implicit by design
  Real& operator+=(Real o) { flopcount::counters().flops += 1; v += o.v; return *this; }
  Real& operator-=(Real o) { flopcount::counters().flops += 1; v -= o.v; return *this; }
  Real& operator*=(Real o) { flopcount::counters().flops += 1; v *= o.v; return *this; }
  Real& operator/=(Real o) { flopcount::counters().flops += 1; v /= o.v; return *this; }
};
inline Real operator+(Real a, Real b) { flopcount::counters().flops += 1; return Real(a.v + b.v); }
inline Real operator-(Real a, Real b) { flopcount::counters().flops += 1; return Real(a.v - b.v); }
inline Real operator*(Real a, Real b) { flopcount::counters().flops += 1; return Real(a.v * b.v); }
inline Real operator/(Real a, Real b) { flopcount::counters().flops += 1; return Real(a.v / b.v); }
inline Real operator-(Real a) { return Real(-a.v); }
inline Real operator+(Real a) { return a; }
inline bool operator<(Real a, Real b) { return a.v < b.v; }
inline bool operator>(Real a, Real b) { return a.v > b.v; }
inline bool operator<=(Real a, Real b) { return a.v <= b.v; }
inline bool operator>=(Real a, Real b) { return a.v >= b.v; }
inline bool operator==(Real a, Real b) { return a.v == b.v; }
inline bool operator!=(Real a, Real b) { return a.v != b.v; }

namespace std {
inline Real fabs(Real a) { return Real(std::fabs(a.v)); }
inline Real sqrt(Real a) { flopcount::counters().flops += 1; return Real(std::sqrt(a.v)); }
inline Real exp(Real a) { flopcount::counters().transcendentals += 1; return Real(std::exp(a.v)); }
inline Real log(Real a) { flopcount::counters().transcendentals += 1; return Real(std::log(a.v)); }
inline Real pow(Real a, Real b) { flopcount::counters().transcendentals += 1; return Real(std::pow(a.v, b.v)); }
inline Real fma(Real a, Real b, Real c) { flopcount::counters().flops += 2; return Real(std::fma(a.v, b.v, c.v)); }
inline bool signbit(Real a) { return std::signbit(a.v); }
inline bool isnan(Real a) { return std::isnan(a.v); }
inline Real max(Real a, Real b) { return a.v < b.v ? b : a; }
inline Real max(double a, Real b) { return a < b.v ? b : Real(a); }
inline Real max(Real a, double b) { return a.v < b ? Real(b) : a; }
inline Real min(Real a, Real b) { return b.v < a.v ? b : a; }
inline Real min(double a, Real b) { return b.v < a ? b : Real(a); }
inline Real min(Real a, double b) { return b < a.v ? Real(b) : a; }
}  // namespace std
