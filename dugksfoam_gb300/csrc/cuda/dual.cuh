// Forward-mode dual number (value, one tangent) for the FP64 tangent-linear
// step: every operation propagates d(x op y) by the chain rule.
#pragma once

#include <cmath>

namespace dugks {

// keep the double overloads visible next to the Dual ones inside this namespace
using ::exp;
using ::fabs;
using ::log;
using ::sqrt;

struct Dual {
    double v, d;
};

__host__ __device__ __forceinline__ Dual dual(double v, double d = 0.0) { return Dual{v, d}; }
__host__ __device__ __forceinline__ Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
__host__ __device__ __forceinline__ Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
__host__ __device__ __forceinline__ Dual operator-(Dual a) { return {-a.v, -a.d}; }
__host__ __device__ __forceinline__ Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
__host__ __device__ __forceinline__ Dual operator/(Dual a, Dual b) {
    const double q = a.v / b.v;
    return {q, (a.d - q * b.d) / b.v};
}
__host__ __device__ __forceinline__ Dual operator+(Dual a, double b) { return {a.v + b, a.d}; }
__host__ __device__ __forceinline__ Dual operator+(double a, Dual b) { return {a + b.v, b.d}; }
__host__ __device__ __forceinline__ Dual operator-(Dual a, double b) { return {a.v - b, a.d}; }
__host__ __device__ __forceinline__ Dual operator-(double a, Dual b) { return {a - b.v, -b.d}; }
__host__ __device__ __forceinline__ Dual operator*(Dual a, double b) { return {a.v * b, a.d * b}; }
__host__ __device__ __forceinline__ Dual operator*(double a, Dual b) { return {a * b.v, a * b.d}; }
__host__ __device__ __forceinline__ Dual operator/(Dual a, double b) { return {a.v / b, a.d / b}; }
__host__ __device__ __forceinline__ Dual operator/(double a, Dual b) {
    const double q = a / b.v;
    return {q, -q * b.d / b.v};
}
__host__ __device__ __forceinline__ Dual& operator+=(Dual& a, Dual b) { a = a + b; return a; }
__host__ __device__ __forceinline__ Dual& operator-=(Dual& a, Dual b) { a = a - b; return a; }
__host__ __device__ __forceinline__ Dual exp(Dual a) {
    const double e = ::exp(a.v);
    return {e, e * a.d};
}
__host__ __device__ __forceinline__ Dual log(Dual a) { return {::log(a.v), a.d / a.v}; }
__host__ __device__ __forceinline__ Dual sqrt(Dual a) {
    const double s = ::sqrt(a.v);
    return {s, 0.5 * a.d / s};
}
__host__ __device__ __forceinline__ Dual fabs(Dual a) { return a.v < 0 ? -a : a; }

}  // namespace dugks
