// gbfem_dual.cuh -- forward-mode dual numbers (value + one directional derivative) for the
// element adjoint. The element math is written once, templated on its scalar type; instantiated
// on Dual it returns, besides each value, the value's derivative along one seeded input
// direction. Comparisons and branches follow the value part, so the derivative is that of the
// branch the value takes (the polar iterations converge quadratically in the derivative too).
#pragma once

#include <cmath>

namespace gbfem {
namespace ad {  // its own namespace: sqrt/fabs below are found by argument-dependent lookup only

struct Dual
{
	double v, d;
	__host__ __device__ Dual(double value = 0.0, double deriv = 0.0) : v(value), d(deriv) {}
	__host__ __device__ explicit operator double() const { return v; }
	__host__ __device__ Dual& operator+=(const Dual& o)
	{
		v += o.v;
		d += o.d;
		return *this;
	}
	__host__ __device__ Dual& operator-=(const Dual& o)
	{
		v -= o.v;
		d -= o.d;
		return *this;
	}
	__host__ __device__ Dual& operator*=(const Dual& o)
	{
		d = d * o.v + v * o.d;
		v *= o.v;
		return *this;
	}
	__host__ __device__ Dual& operator/=(const Dual& o)
	{
		const double q = v / o.v;
		d = (d - q * o.d) / o.v;
		v = q;
		return *this;
	}
};

__host__ __device__ inline Dual operator+(const Dual& a, const Dual& b) { return Dual(a.v + b.v, a.d + b.d); }
__host__ __device__ inline Dual operator-(const Dual& a, const Dual& b) { return Dual(a.v - b.v, a.d - b.d); }
__host__ __device__ inline Dual operator-(const Dual& a) { return Dual(-a.v, -a.d); }
__host__ __device__ inline Dual operator*(const Dual& a, const Dual& b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__host__ __device__ inline Dual operator/(const Dual& a, const Dual& b)
{
	const double q = a.v / b.v;
	return Dual(q, (a.d - q * b.d) / b.v);
}
__host__ __device__ inline bool operator<(const Dual& a, const Dual& b) { return a.v < b.v; }
__host__ __device__ inline bool operator>(const Dual& a, const Dual& b) { return a.v > b.v; }
__host__ __device__ inline bool operator<=(const Dual& a, const Dual& b) { return a.v <= b.v; }
__host__ __device__ inline bool operator>=(const Dual& a, const Dual& b) { return a.v >= b.v; }
__host__ __device__ inline bool operator==(const Dual& a, const Dual& b) { return a.v == b.v; }
__host__ __device__ inline bool operator!=(const Dual& a, const Dual& b) { return a.v != b.v; }
__host__ __device__ inline Dual sqrt(const Dual& a)
{
	const double s = ::sqrt(a.v);
	return Dual(s, s > 0.0 ? a.d / (2.0 * s) : 0.0);
}
__host__ __device__ inline Dual fabs(const Dual& a) { return a.v < 0.0 ? -a : a; }

}  // namespace ad
using ad::Dual;
}  // namespace gbfem
