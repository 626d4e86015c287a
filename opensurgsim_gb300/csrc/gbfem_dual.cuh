// gbfem_dual.cuh -- forward-mode dual numbers (value + one directional derivative) for the
// element adjoint. The element math is written once, templated on its scalar type; instantiated
// on a dual type it returns, besides each value, the value's derivative along one seeded input
// direction. Comparisons and branches follow the value part, so the derivative is that of the
// branch the value takes (the polar iterations converge quadratically in the derivative too).
// DualT<double> serves the FP64 form, DualT<float> the mixed form.
#pragma once

#include <cmath>

namespace gbfem {
namespace ad {  // its own namespace: sqrt/fabs below are found by argument-dependent lookup only

template <typename S>
struct DualT
{
	S v, d;
	__host__ __device__ DualT(double value = 0.0, double deriv = 0.0) : v(S(value)), d(S(deriv)) {}
	__host__ __device__ explicit operator double() const { return double(v); }
	__host__ __device__ DualT& operator+=(const DualT& o)
	{
		v += o.v;
		d += o.d;
		return *this;
	}
	__host__ __device__ DualT& operator-=(const DualT& o)
	{
		v -= o.v;
		d -= o.d;
		return *this;
	}
	__host__ __device__ DualT& operator*=(const DualT& o)
	{
		d = d * o.v + v * o.d;
		v *= o.v;
		return *this;
	}
	__host__ __device__ DualT& operator/=(const DualT& o)
	{
		const S q = v / o.v;
		d = (d - q * o.d) / o.v;
		v = q;
		return *this;
	}
	__host__ __device__ static DualT make(S value, S deriv)
	{
		DualT r;
		r.v = value;
		r.d = deriv;
		return r;
	}
};

template <typename S>
__host__ __device__ inline DualT<S> operator+(const DualT<S>& a, const DualT<S>& b)
{
	return DualT<S>::make(a.v + b.v, a.d + b.d);
}
template <typename S>
__host__ __device__ inline DualT<S> operator-(const DualT<S>& a, const DualT<S>& b)
{
	return DualT<S>::make(a.v - b.v, a.d - b.d);
}
template <typename S>
__host__ __device__ inline DualT<S> operator-(const DualT<S>& a)
{
	return DualT<S>::make(-a.v, -a.d);
}
template <typename S>
__host__ __device__ inline DualT<S> operator*(const DualT<S>& a, const DualT<S>& b)
{
	return DualT<S>::make(a.v * b.v, a.d * b.v + a.v * b.d);
}
template <typename S>
__host__ __device__ inline DualT<S> operator/(const DualT<S>& a, const DualT<S>& b)
{
	const S q = a.v / b.v;
	return DualT<S>::make(q, (a.d - q * b.d) / b.v);
}
// Mixed operands: a plain number is a constant (zero derivative), so only the parts that carry a
// derivative are computed (the same values as promoting it to a dual, without the products and sums
// with a zero derivative). The plain operand converts to S (a non-deduced parameter).
template <typename S>
struct Plain
{
	using type = S;
};
template <typename S>
using PlainT = typename Plain<S>::type;
template <typename S>
__host__ __device__ inline DualT<S> operator+(const DualT<S>& a, PlainT<S> b) { return DualT<S>::make(a.v + b, a.d); }
template <typename S>
__host__ __device__ inline DualT<S> operator+(PlainT<S> a, const DualT<S>& b) { return DualT<S>::make(a + b.v, b.d); }
template <typename S>
__host__ __device__ inline DualT<S> operator-(const DualT<S>& a, PlainT<S> b) { return DualT<S>::make(a.v - b, a.d); }
template <typename S>
__host__ __device__ inline DualT<S> operator-(PlainT<S> a, const DualT<S>& b) { return DualT<S>::make(a - b.v, -b.d); }
template <typename S>
__host__ __device__ inline DualT<S> operator*(const DualT<S>& a, PlainT<S> b) { return DualT<S>::make(a.v * b, a.d * b); }
template <typename S>
__host__ __device__ inline DualT<S> operator*(PlainT<S> a, const DualT<S>& b) { return DualT<S>::make(a * b.v, a * b.d); }
template <typename S>
__host__ __device__ inline DualT<S> operator/(const DualT<S>& a, PlainT<S> b) { return DualT<S>::make(a.v / b, a.d / b); }
template <typename S>
__host__ __device__ inline DualT<S> operator/(PlainT<S> a, const DualT<S>& b)
{
	const S q = a / b.v;
	return DualT<S>::make(q, -(q * b.d) / b.v);
}
template <typename S>
__host__ __device__ inline bool operator<(const DualT<S>& a, const DualT<S>& b) { return a.v < b.v; }
template <typename S>
__host__ __device__ inline bool operator>(const DualT<S>& a, const DualT<S>& b) { return a.v > b.v; }
template <typename S>
__host__ __device__ inline bool operator<=(const DualT<S>& a, const DualT<S>& b) { return a.v <= b.v; }
template <typename S>
__host__ __device__ inline bool operator>=(const DualT<S>& a, const DualT<S>& b) { return a.v >= b.v; }
template <typename S>
__host__ __device__ inline bool operator==(const DualT<S>& a, const DualT<S>& b) { return a.v == b.v; }
template <typename S>
__host__ __device__ inline bool operator!=(const DualT<S>& a, const DualT<S>& b) { return a.v != b.v; }
template <typename S>
__host__ __device__ inline bool operator<(const DualT<S>& a, double b) { return a.v < b; }
template <typename S>
__host__ __device__ inline bool operator>(const DualT<S>& a, double b) { return a.v > b; }
template <typename S>
__host__ __device__ inline DualT<S> sqrt(const DualT<S>& a)
{
	const S s = ::sqrt(a.v);
	return DualT<S>::make(s, s > S(0) ? a.d / (S(2) * s) : S(0));
}
template <typename S>
__host__ __device__ inline DualT<S> fabs(const DualT<S>& a)
{
	return a.v < S(0) ? -a : a;
}

}  // namespace ad
using Dual = ad::DualT<double>;
using DualF = ad::DualT<float>;
}  // namespace gbfem
