// Forward-mode dual number (value, derivative) for the tangent-linear step.
//
// Instantiating the exact tile body with Dual gives the tangent-linear model of
// the advance with no hand-written derivative code: every operation carries its
// derivative by the chain rule, branches follow the value.  It is the
// independent reference the hand-written adjoint is checked against
// (<J v, w> == <v, J^T w>).
#pragma once

#include <cmath>

namespace hx {

struct Dual {
    double v, d;
    __host__ __device__ constexpr Dual() : v(0.0), d(0.0) {}
    __host__ __device__ constexpr Dual(double x) : v(x), d(0.0) {}
    __host__ __device__ constexpr Dual(double x, double y) : v(x), d(y) {}
    __host__ __device__ explicit operator double() const { return v; }

    __host__ __device__ friend Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
    __host__ __device__ friend Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
    __host__ __device__ friend Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
    __host__ __device__ friend Dual operator/(Dual a, Dual b) {
        const double q = a.v / b.v;
        return Dual(q, (a.d - q * b.d) / b.v);
    }
    __host__ __device__ friend Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
    __host__ __device__ Dual& operator+=(Dual b) { v += b.v; d += b.d; return *this; }
    __host__ __device__ Dual& operator-=(Dual b) { v -= b.v; d -= b.d; return *this; }
    __host__ __device__ Dual& operator*=(Dual b) { *this = *this * b; return *this; }

    __host__ __device__ friend bool operator<(Dual a, Dual b) { return a.v < b.v; }
    __host__ __device__ friend bool operator>(Dual a, Dual b) { return a.v > b.v; }
    __host__ __device__ friend bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
    __host__ __device__ friend bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
    __host__ __device__ friend bool operator==(Dual a, Dual b) { return a.v == b.v; }
    __host__ __device__ friend bool operator!=(Dual a, Dual b) { return a.v != b.v; }

    // found by argument-dependent lookup only, so ::sqrt(double) stays visible
    __host__ __device__ friend Dual sqrt(Dual a) {
        const double s = ::sqrt(a.v);
        return Dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
    }
    __host__ __device__ friend Dual cbrt(Dual a) {
        const double c = ::cbrt(a.v);
        return Dual(c, c != 0.0 ? a.d / (3.0 * c * c) : 0.0);
    }
    __host__ __device__ friend Dual fabs(Dual a) {
        return a.v > 0.0 ? a : (a.v < 0.0 ? -a : Dual(0.0, 0.0));
    }
    __host__ __device__ friend bool isnan(Dual a) { return a.v != a.v; }
};

}  // namespace hx
