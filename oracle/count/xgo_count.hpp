// xgo_count.hpp — a counting FP64 scalar for the oracle (TEST INFRASTRUCTURE
// ONLY).  oracle/count/xgo_count.cpp compiles the oracle's C sources as C++
// with every `double` replaced by `xcnt`, so one load of a circuit counts the
// floating-point operations the reference's device equations perform (the
// algorithmic flops of the load), by kind, along the branches each instance
// takes on its own inputs.  An xcnt is one double in memory, so the oracle's
// arrays and structures keep their layout and take plain double buffers.
#ifndef XGO_COUNT_HPP
#define XGO_COUNT_HPP

#include <ctype.h>
#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <type_traits>

enum { XC_ADD, XC_MUL, XC_DIV, XC_SQRT, XC_EXP, XC_LOG, XC_NKIND };
extern "C" unsigned long long xgo_count_ops[XC_NKIND];

struct xcnt {
  double v;
  xcnt() = default;
  template <class T, class = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  constexpr xcnt(T x) : v((double)x) {}
  template <class T, class = typename std::enable_if<std::is_arithmetic<T>::value>::type>
  explicit operator T() const { return (T)v; }
};
static_assert(sizeof(xcnt) == sizeof(double), "xcnt must have the layout of a double");

inline xcnt xc_op(int kind, double r) {
  ++xgo_count_ops[kind];
  return xcnt(r);
}
template <class T>
struct xc_num {
  static constexpr bool value = std::is_arithmetic<T>::value || std::is_enum<T>::value;
};
template <class T>
using xc_arith = typename std::enable_if<xc_num<T>::value, xcnt>::type;
template <class T>
using xc_bool = typename std::enable_if<xc_num<T>::value, bool>::type;

inline xcnt operator+(xcnt a, xcnt b) { return xc_op(XC_ADD, a.v + b.v); }
inline xcnt operator-(xcnt a, xcnt b) { return xc_op(XC_ADD, a.v - b.v); }
inline xcnt operator*(xcnt a, xcnt b) { return xc_op(XC_MUL, a.v * b.v); }
inline xcnt operator/(xcnt a, xcnt b) { return xc_op(XC_DIV, a.v / b.v); }
template <class T> xc_arith<T> operator+(xcnt a, T b) { return a + xcnt(b); }
template <class T> xc_arith<T> operator-(xcnt a, T b) { return a - xcnt(b); }
template <class T> xc_arith<T> operator*(xcnt a, T b) { return a * xcnt(b); }
template <class T> xc_arith<T> operator/(xcnt a, T b) { return a / xcnt(b); }
template <class T> xc_arith<T> operator+(T a, xcnt b) { return xcnt(a) + b; }
template <class T> xc_arith<T> operator-(T a, xcnt b) { return xcnt(a) - b; }
template <class T> xc_arith<T> operator*(T a, xcnt b) { return xcnt(a) * b; }
template <class T> xc_arith<T> operator/(T a, xcnt b) { return xcnt(a) / b; }
inline xcnt operator-(xcnt a) { return xcnt(-a.v); }  // a sign flip, not an operation
inline xcnt operator+(xcnt a) { return a; }
inline xcnt &operator+=(xcnt &a, xcnt b) { return a = a + b; }
inline xcnt &operator-=(xcnt &a, xcnt b) { return a = a - b; }
inline xcnt &operator*=(xcnt &a, xcnt b) { return a = a * b; }
inline xcnt &operator/=(xcnt &a, xcnt b) { return a = a / b; }

#define XC_CMP(op)                                                          \
  inline bool operator op(xcnt a, xcnt b) { return a.v op b.v; }            \
  template <class T> xc_bool<T> operator op(xcnt a, T b) { return a.v op (double)b; } \
  template <class T> xc_bool<T> operator op(T a, xcnt b) { return (double)a op b.v; }
XC_CMP(<)
XC_CMP(>)
XC_CMP(<=)
XC_CMP(>=)
XC_CMP(==)
XC_CMP(!=)
#undef XC_CMP
inline bool operator!(xcnt a) { return !a.v; }

inline xcnt sqrt(xcnt a) { return xc_op(XC_SQRT, ::sqrt(a.v)); }
inline xcnt exp(xcnt a) { return xc_op(XC_EXP, ::exp(a.v)); }
inline xcnt log(xcnt a) { return xc_op(XC_LOG, ::log(a.v)); }
inline xcnt fabs(xcnt a) { return xcnt(::fabs(a.v)); }     // sign clear
inline xcnt floor(xcnt a) { return xcnt(::floor(a.v)); }   // rounding, not arithmetic

#endif
