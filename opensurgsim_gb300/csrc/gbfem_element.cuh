// gbfem_element.cuh -- per-element corotational-tetrahedron math, templated on the arithmetic
// type of the bulk work (double for the plain form, float for the mixed form, Dual for the
// element derivatives of the adjoint).
//
// Closed form on the shape-function gradients g_a (rows of V^-1) instead of 12x12 products.
// With h_a = R g_a and G_ab = g_a . g_b:
//   K0_ab   = V (lambda g_a g_b^T + mu g_b g_a^T + mu G_ab I)            (= V B^T Em B)
//   Krot_ab = V (lambda h_a h_b^T + mu h_b h_a^T + mu G_ab I)            (= R K0_ab R^T)
//   dR/dx_(b,q) = [psi_bq]x R,  psi_bq = G^-1 (g_b x r_q),  r_q = row q of R
//   extra(3a+i, 3b+q) = (T_a G^-1 (g_b x r_q))_i,
//   T_a = -[R y_a]x + R (sum_c K0_ac [w_c]x) R^T,  w_c = R^T (x_c - x_0) - (x0_c - x0_0),
//   y = Krot w  (the reference's KTimesRx_x0, Fem3DElementCorotationalTetrahedron.cpp:276,
//   which multiplies by the rotated stiffness rather than K0),
// so that K_e = Krot + extra reproduces Fem3DElementCorotationalTetrahedron.cpp:199-286 and
// f_e = -K_e (x - R x0) = -(R K0 w + T' zeta) reproduces :103-113. All quantities use positions
// relative to node 0 (the tangent annihilates translations). The corotated strain w never comes
// from plain FP32 differences, which would lose |strain|/eps32 of its digits: the FP64 form takes
// it from FP64 edges, the FP32 form from Gram differences p.p - q.q formed in double-float
// arithmetic on float-pair positions (gram_diff below).
#pragma once

#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "gbfem_dual.cuh"
#include "gbfem_internal.h"

namespace gbfem {
namespace elem {

// Knuth's TwoSum in FP32: a + b = s + e exactly. The _rn intrinsics keep the compiler from
// contracting or reassociating it.
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

template <typename T>
__host__ __device__ __forceinline__ void cofactor3(const T* X, T* C)
{
	C[0] = X[4] * X[8] - X[5] * X[7];
	C[1] = X[5] * X[6] - X[3] * X[8];
	C[2] = X[3] * X[7] - X[4] * X[6];
	C[3] = X[2] * X[7] - X[1] * X[8];
	C[4] = X[0] * X[8] - X[2] * X[6];
	C[5] = X[1] * X[6] - X[0] * X[7];
	C[6] = X[1] * X[5] - X[2] * X[4];
	C[7] = X[2] * X[3] - X[0] * X[5];
	C[8] = X[0] * X[4] - X[1] * X[3];
}

template <typename T>
__host__ __device__ __forceinline__ T det3(const T* X)
{
	return X[0] * (X[4] * X[8] - X[5] * X[7]) - X[1] * (X[3] * X[8] - X[5] * X[6]) + X[2] * (X[3] * X[7] - X[4] * X[6]);
}

template <typename A, typename B, typename T>
__host__ __device__ __forceinline__ void cross3(const A* a, const B* b, T* c)
{
	c[0] = a[1] * b[2] - a[2] * b[1];
	c[1] = a[2] * b[0] - a[0] * b[2];
	c[2] = a[0] * b[1] - a[1] * b[0];
}

template <typename T>
struct Eps;
template <>
struct Eps<double>
{
	static constexpr double eps = DBL_EPSILON;
	static constexpr double newtonTol2 = 1e-26;  // |X_k+1 - X_k|_F^2 at convergence
};
template <>
struct Eps<float>
{
	static constexpr float eps = FLT_EPSILON;
	static constexpr float newtonTol2 = 1e-11f;
};
template <>
struct Eps<Dual>
{
	static constexpr double eps = DBL_EPSILON;
	static constexpr double newtonTol2 = 1e-26;
};
template <>
struct Eps<DualF>
{
	static constexpr double eps = FLT_EPSILON;
	static constexpr double newtonTol2 = 1e-11;
};

// The plain scalar under an arithmetic type: itself, or the value type of a dual number. The rest
// shape, the moduli and the inputs other than the positions enter compute() as plain scalars.
template <typename T>
struct ScalarOf
{
	using type = T;
};
template <typename S>
struct ScalarOf<ad::DualT<S>>
{
	using type = S;
};
template <typename T>
struct IsDual : std::false_type
{
};
template <typename S>
struct IsDual<ad::DualT<S>> : std::true_type
{
};

// Polar factor by Newton's iteration X <- (g X + X^-T / g) / 2 (Higham), Frobenius scaling on the
// first iterations. Valid for det F > 0, where the orthogonal polar factor is the rotation that
// Transform::computeRotationScaling returns. Returns false (the caller falls back to the SVD) for
// det F <= 0 (FP32: det F <= 1e-5 |F|_F^3) or when the iteration does not settle within its bound.
template <typename T>
__host__ __device__ bool polar_newton(const T* F, T* R)
{
	T X[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) X[k] = F[k];
	for (int it = 0; it < 20; ++it)
	{
		T C[9];
		cofactor3(X, C);
		const T d = X[0] * C[0] + X[1] * C[1] + X[2] * C[2];
		if (!(d > T(0))) return false;
		T gam = T(1);
		if (it < 3)
		{
			T nx = 0, nc = 0;
#pragma unroll
			for (int k = 0; k < 9; ++k)
			{
				nx += X[k] * X[k];
				nc += C[k] * C[k];
			}
			// FP32: a nearly degenerate F (det F below 1e-5 of |F|_F^3) goes to the FP64 SVD path, where
			// a collapsed element's singular G is decided in FP64 as the reference decides it.
			if (std::is_same<T, float>::value && it == 0 && !(d > T(1e-5) * nx * sqrt(nx))) return false;
			gam = sqrt(sqrt(nc / (nx * d * d)));
		}
		const T a = T(0.5) * gam;
		const T b = T(0.5) / (gam * d);
		T diff = 0;
#pragma unroll
		for (int k = 0; k < 9; ++k)
		{
			const T xn = a * X[k] + b * C[k];
			const T dd = xn - X[k];
			diff += dd * dd;
			X[k] = xn;
		}
		if (diff < Eps<T>::newtonTol2 && it >= 1)
		{
#pragma unroll
			for (int k = 0; k < 9; ++k) R[k] = X[k];
			return true;
		}
	}
	return false;
}

// SVD-based polar factor for any F (one-sided Jacobi, bounded sweeps): proper rotation with the
// reflection placed on the smallest singular value, R = U diag(1,1,det(U V^T)) V^T. sig (optional)
// receives the eigenvalues of S = R^T F, the singular values with that sign on the smallest.
template <typename T>
__host__ __device__ void polar_svd(const T* F, T* R, T* sig = nullptr)
{
	T A[9], V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
#pragma unroll
	for (int k = 0; k < 9; ++k) A[k] = F[k];
	for (int sweep = 0; sweep < 40; ++sweep)
	{
		bool rotated = false;
		for (int pp = 0; pp < 3; ++pp)
		{
			const int p = (pp == 2) ? 1 : 0;
			const int q = (pp == 0) ? 1 : 2;
			T al = 0, be = 0, ga = 0;
			for (int k = 0; k < 3; ++k)
			{
				al += A[3 * k + p] * A[3 * k + p];
				be += A[3 * k + q] * A[3 * k + q];
				ga += A[3 * k + p] * A[3 * k + q];
			}
			if (ga == T(0) || fabs(ga) <= Eps<T>::eps * sqrt(al * be)) continue;
			rotated = true;
			const T zeta = (be - al) / (T(2) * ga);
			const T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
			const T c = T(1) / sqrt(T(1) + t * t);
			const T s = c * t;
			for (int k = 0; k < 3; ++k)
			{
				const T ap = A[3 * k + p], aq = A[3 * k + q];
				A[3 * k + p] = c * ap - s * aq;
				A[3 * k + q] = s * ap + c * aq;
				const T vp = V[3 * k + p], vq = V[3 * k + q];
				V[3 * k + p] = c * vp - s * vq;
				V[3 * k + q] = s * vp + c * vq;
			}
		}
		if (!rotated) break;
	}
	T sv[3];
	for (int j = 0; j < 3; ++j) sv[j] = sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
	int o[3] = {0, 1, 2};
	if (sv[o[0]] < sv[o[1]]) { const int tt = o[0]; o[0] = o[1]; o[1] = tt; }
	if (sv[o[1]] < sv[o[2]]) { const int tt = o[1]; o[1] = o[2]; o[2] = tt; }
	if (sv[o[0]] < sv[o[1]]) { const int tt = o[0]; o[0] = o[1]; o[1] = tt; }
	T U[9], Vs[9];
	for (int j = 0; j < 3; ++j)
		for (int k = 0; k < 3; ++k) Vs[3 * k + j] = V[3 * k + o[j]];
	const T smax = sv[o[0]] > T(0) ? sv[o[0]] : T(1);
	for (int j = 0; j < 3; ++j)
	{
		const T s = sv[o[j]];
		if (s > T(1e-12) * smax && s > T(0))
		{
			for (int k = 0; k < 3; ++k) U[3 * k + j] = A[3 * k + o[j]] / s;
		}
		else if (j == 2)
		{
			U[2] = U[3] * U[7] - U[6] * U[4];
			U[5] = U[6] * U[1] - U[0] * U[7];
			U[8] = U[0] * U[4] - U[3] * U[1];
		}
		else
		{
			// Rank < 2: complete with the canonical axis least aligned with column 0.
			int ax = 0;
			T best = T(2);
			for (int a = 0; a < 3; ++a)
			{
				const T d = (j == 0) ? T(0) : fabs(U[3 * a]);
				if (d < best)
				{
					best = d;
					ax = a;
				}
			}
			T e[3] = {T(ax == 0), T(ax == 1), T(ax == 2)};
			if (j == 1)
			{
				const T d = e[0] * U[0] + e[1] * U[3] + e[2] * U[6];
				for (int k = 0; k < 3; ++k) e[k] -= d * U[3 * k];
			}
			const T nrm = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
			for (int k = 0; k < 3; ++k) U[3 * k + j] = e[k] / nrm;
		}
	}
	const T x = (det3(U) * det3(Vs) < T(0)) ? T(-1) : T(1);
	for (int k = 0; k < 3; ++k) U[3 * k + 2] *= x;
	if (sig)
	{
		sig[0] = sv[o[0]];
		sig[1] = sv[o[1]];
		sig[2] = x * sv[o[2]];
	}
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
			R[3 * i + j] = U[3 * i] * Vs[3 * j] + U[3 * i + 1] * Vs[3 * j + 1] + U[3 * i + 2] * Vs[3 * j + 2];
}

// (K0 u)_a = lambdaV tr(D) g_a + muV D^T g_a + muV sum_c G_ac u_c,  D = sum_c u_c g_c^T.
template <typename T, typename G>
__host__ __device__ __forceinline__ void k0_apply(const G (&g)[4][3], const G (&Gab)[4][4], G lamV, G muV, const T (&u)[4][3],
										 T (&out)[4][3])
{
	T D[3][3];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) D[i][j] = u[0][i] * g[0][j] + u[1][i] * g[1][j] + u[2][i] * g[2][j] + u[3][i] * g[3][j];
	const T tr = D[0][0] + D[1][1] + D[2][2];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int j = 0; j < 3; ++j)
			out[a][j] = lamV * tr * g[a][j] + muV * (D[0][j] * g[a][0] + D[1][j] * g[a][1] + D[2][j] * g[a][2]) +
						muV * (Gab[a][0] * u[0][j] + Gab[a][1] * u[1][j] + Gab[a][2] * u[2][j] + Gab[a][3] * u[3][j]);
}

__host__ __device__ __forceinline__ int pair_slot(int a, int b)
{
	// (0,1)->4 (0,2)->5 (0,3)->6 (1,2)->7 (1,3)->8 (2,3)->9 for a < b
	return (a == 0) ? (3 + b) : (a == 1 ? (5 + b) : 9);
}

// Per-element inputs gathered by the kernels (node 0 is the origin of p and q). The positions p have
// scalar type P (double, or a dual type when the adjoint seeds a derivative direction in them); the
// other inputs never carry a derivative and have type C (double, or the dual passes' plain type).
template <typename P, typename C = double>
struct ElemInT
{
	int nd[4];
	P p[4][3];    // x_n,a - x_n,0
	C q[4][3];    // x0_a - x0_0
	C uK[4][3];   // -beta v_n + (x_n - x_t - dt v_n)
	C uM[4][3];   // -alpha v_n - (v_n - v_t)/dt
	C vv[4][3];   // v_n (debug force only)
	double alphaDbg, betaDbg;  // Rayleigh coefficients (debug force only)
	int lumped = 0;  // FemRepresentation::setMassLumping: the element's mass rows summed onto the diagonal
};
using ElemIn = ElemInT<double>;

__device__ __forceinline__ void gather(const DevBody& b, int e, const double* __restrict__ xn,
									   const double* __restrict__ vn, const double* __restrict__ xt,
									   const double* __restrict__ vt, double dt, double alpha, double beta, ElemIn& in)
{
	const int4 t4 = b.tets[e];
	in.nd[0] = t4.x;
	in.nd[1] = t4.y;
	in.nd[2] = t4.z;
	in.nd[3] = t4.w;
	double x0[3], r0[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		x0[k] = xn[3 * in.nd[0] + k];
		r0[k] = b.xrest[3 * in.nd[0] + k];
	}
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			const int d = 3 * in.nd[a] + k;
			const double xa = xn[d], va = vn[d];
			in.p[a][k] = xa - x0[k];
			in.q[a][k] = b.xrest[d] - r0[k];
			in.uK[a][k] = -beta * va + ((xa - xt[d]) - dt * va);
			in.uM[a][k] = -alpha * va - (va - vt[d]) / dt;
			in.vv[a][k] = va;
		}
	in.alphaDbg = alpha;
	in.betaDbg = beta;
	in.lumped = b.lumped;
}

// Inputs of the FP32 element kernel. FP64 issues at 1/64 of the FP32 rate here, so the corotational
// kernel runs no FP64 at all: its per-node inputs come from the node pass (k_node_prep) in FP32,
// positions as unevaluated float pairs hi + lo (~2^-48 relative), and the edges relative to node 0
// and the Gram differences of the strain are formed in double-float arithmetic. The right-hand-side
// inputs are FP32 differences x_n - x_t, v_n - v_t (zero, and not read, in the first Newton
// iteration). The linear tetrahedron keeps FP64 edges p and rest edges q (its strain needs no Gram).
struct ElemInF
{
	int nd[4];
	double p[4][3];   // x_n,a - x_n,0 (linear tetrahedra)
	double q[4][3];   // x0_a - x0_0 (linear tetrahedra)
	float ph[4][3];   // corotational: x_n,a - x_n,0 as a float pair ph + pl
	float pl[4][3];
	// Corotational: the element's precomputed rest edges (FP32, [3(a-1)+k][E]) and rest Gram
	// q_a . q_c as float pairs ([(a,c)][E]), read where they are used.
	const float* qf32;
	const float2* qg2;
	int E, e;
	float uK[4][3];   // (x_n - x_t) - (beta + dt) v_n
	float uM[4][3];   // -alpha v_n - (v_n - v_t) / dt
	float vv[4][3];   // v_n (debug force only; unused by the FP32 kernel)
	double alphaDbg, betaDbg;
	int lumped = 0;   // mass lumping (as ElemInT::lumped)
};

// kLinear: p and q in FP64 from the positions and rest positions (u = x - x0 is formed from them).
// Corotational: FP32 node-pass values only (x as float pairs, v, and the differences to the step's
// start state); the rest edges (FP32) and rest Gram (float pairs) are precomputed per element, so
// rest positions are not gathered.
template <bool kLinear>
__device__ __forceinline__ void gather_f32(const DevBody& b, int e, const double* __restrict__ xn,
										   const double* __restrict__ vn, const double* __restrict__ xt,
										   const double* __restrict__ vt, float c2, float alpha, float inv_dt,
										   ElemInF& in)
{
	const bool startState = (xt == xn) && (vt == vn);  // uniform over the grid
	const int4 t4 = b.tets[e];
	in.nd[0] = t4.x;
	in.nd[1] = t4.y;
	in.nd[2] = t4.z;
	in.nd[3] = t4.w;
	in.qf32 = b.qf32;
	in.qg2 = b.qg2;
	in.E = b.E;
	in.e = e;
	if constexpr (!kLinear)
	{
		// Node pass outputs: x as (hi, lo), v, and x_n - x_t, v_n - v_t past the first Newton iteration.
		float xh[4][3], xl[4][3];
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				const int d = 3 * in.nd[a] + k;
				const float2 xp = b.nodeX[d];
				xh[a][k] = xp.x;
				xl[a][k] = xp.y;
				const float vf = b.nodeV[d];
				if (startState)
				{
					in.uK[a][k] = -c2 * vf;
					in.uM[a][k] = -alpha * vf;
				}
				else
				{
					in.uK[a][k] = __fmaf_rn(-c2, vf, b.nodeDx[d]);
					in.uM[a][k] = -alpha * vf - b.nodeDv[d] * inv_dt;
				}
				in.vv[a][k] = vf;
			}
		// Edge a: (xh_a - xh_0) exactly as a TwoSum pair, plus (xl_a - xl_0), renormalised.
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			in.ph[0][k] = 0.f;
			in.pl[0][k] = 0.f;
		}
#pragma unroll
		for (int a = 1; a < 4; ++a)
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				float s, es;
				df_two_sum(xh[a][k], -xh[0][k], s, es);
				df_two_sum(s, __fadd_rn(es, __fsub_rn(xl[a][k], xl[0][k])), in.ph[a][k], in.pl[a][k]);
			}
	}
	else
	{
		double x0[3], r0[3];
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			x0[k] = xn[3 * in.nd[0] + k];
			r0[k] = b.xrest[3 * in.nd[0] + k];
		}
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				const int d = 3 * in.nd[a] + k;
				const double xa = xn[d], va = vn[d];
				in.p[a][k] = xa - x0[k];
				in.q[a][k] = b.xrest[d] - r0[k];
				const float vf = float(va);
				if (startState)
				{
					in.uK[a][k] = -c2 * vf;
					in.uM[a][k] = -alpha * vf;
				}
				else
				{
					in.uK[a][k] = __fmaf_rn(-c2, vf, float(xa - xt[d]));
					in.uM[a][k] = -alpha * vf - float(va - vt[d]) * inv_dt;
				}
				in.vv[a][k] = vf;
			}
	}
	in.alphaDbg = 0.0;
	in.betaDbg = 0.0;
	in.lumped = b.lumped;
}

// Rest Gram entry q_a . q_c (a <= c, both in 1..3) and rest edge components for the FP32 strain:
// precomputed in the mixed kernel's input, formed from the rest positions otherwise.
__host__ __device__ __forceinline__ int gram_index(int a, int c)
{
	return (a == 1) ? (c - 1) : (a == 2 ? 1 + c : 5);  // (1,1) (1,2) (1,3) (2,2) (2,3) (3,3)
}
template <typename In>
__host__ __device__ __forceinline__ double rest_gram(const In& in, int a, int c)
{
	const auto* qa = in.q[a];
	const auto* qc = in.q[c];
	return double(qa[0]) * double(qc[0]) + double(qa[1]) * double(qc[1]) + double(qa[2]) * double(qc[2]);
}
// Gram difference p_a . p_c - q_a . q_c (a, c in 1..3), rounded to FP32 at the end: from FP64 edges,
// or, for the corotational FP32 kernel, in double-float (each product's rounding error by FMA, the
// sums by TwoSum, the rest Gram as a float pair), so the cancellation between the two Grams of a
// rotated, barely strained element keeps the strain to FP32 relative accuracy with no FP64.
template <typename In>
__host__ __device__ __forceinline__ float gram_diff(const In& in, int a, int c)
{
	const double* pa = in.p[a];
	const double* pc = in.p[c];
	return float((pa[0] * pc[0] + pa[1] * pc[1] + pa[2] * pc[2]) - rest_gram(in, a, c));
}
__device__ __forceinline__ float gram_diff(const ElemInF& in, int a, int c)
{
	float sh = 0.f, sl = 0.f;
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		const float P = __fmul_rn(in.ph[a][k], in.ph[c][k]);
		const float e = __fmaf_rn(in.ph[a][k], in.ph[c][k], -P);
		const float cross = __fmaf_rn(in.ph[a][k], in.pl[c][k], __fmul_rn(in.pl[a][k], in.ph[c][k]));
		float t, et;
		df_two_sum(sh, P, t, et);
		sh = t;
		sl = __fadd_rn(sl, __fadd_rn(et, __fadd_rn(e, cross)));
	}
	const float2 q = in.qg2[(size_t)gram_index(a, c) * in.E + in.e];
	float d, ed;
	df_two_sum(sh, -q.x, d, ed);
	return __fadd_rn(d, __fadd_rn(ed, __fsub_rn(sl, q.y)));
}
// Edge a of the element (x_a - x_0), component i, in the kernel's type.
template <typename T, bool kLinear, typename In>
__host__ __device__ __forceinline__ T edge(const In& in, int a, int i)
{
	return T(in.p[a][i]);
}
template <typename T, bool kLinear>
__host__ __device__ __forceinline__ T edge(const ElemInF& in, int a, int i)
{
	if constexpr (kLinear)
		return T(in.p[a][i]);
	else
		return T(in.ph[a][i]) + T(in.pl[a][i]);
}
template <typename In>
__host__ __device__ __forceinline__ float rest_edge(const In& in, int a, int k)
{
	return float(in.q[a][k]);
}
__host__ __device__ __forceinline__ float rest_edge(const ElemInF& in, int a, int k)
{
	return a == 0 ? 0.f : in.qf32[(size_t)(3 * (a - 1) + k) * in.E + in.e];
}

// F = sum_a p_a g_a^T (linear part of P V^-1, Fem3DElementCorotationalTetrahedron.cpp:146).
template <typename T, bool kLinear, typename In>
__host__ __device__ __forceinline__ void deformation(const In& in, const typename ScalarOf<T>::type (&g)[4][3], T (&F)[9])
{
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
			F[3 * i + j] = edge<T, kLinear>(in, 1, i) * g[1][j] + edge<T, kLinear>(in, 2, i) * g[2][j] +
						   edge<T, kLinear>(in, 3, i) * g[3][j];
}

// The element's rotation R (row-major, F = R S) from its deformation gradient F: Newton's polar
// iteration, the SVD path for near-inverted or degenerate elements (always at least FP64), the
// identity for the linear tetrahedron. Returns flags 1 (SVD path) and 4 (the FP32 form's FP64
// singular-G decision on that path) of compute_to().
template <typename T, bool kLinear, typename In>
__host__ __device__ __forceinline__ int rotation(const In& in, const typename ScalarOf<T>::type (&g)[4][3], const T (&F)[9],
												 T (&R)[9])
{
	int flags = 0;
	if constexpr (kLinear)
	{
#pragma unroll
		for (int k = 0; k < 9; ++k) R[k] = (k % 4 == 0) ? T(1) : T(0);
	}
	else if (!polar_newton(F, R))
	{
		// Near-inverted or degenerate element: SVD path (the reference's computeRotationScaling),
		// always at least FP64.
		if constexpr (std::is_same<T, float>::value)
		{
			double Fd[9], Rd[9], sg[3];
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
					Fd[3 * i + j] = edge<double, kLinear>(in, 1, i) * double(g[1][j]) +
									edge<double, kLinear>(in, 2, i) * double(g[2][j]) +
									edge<double, kLinear>(in, 3, i) * double(g[3][j]);
			polar_svd(Fd, Rd, sg);
#pragma unroll
			for (int k = 0; k < 9; ++k) R[k] = T(Rd[k]);
			// The reference's singular-G test is absolute (|det G| <= 1e-12, :210), below what the
			// FP32 G resolves (its entries carry ~1e-7 of rounding). On this path it is decided in
			// FP64: det G = det(tr(S) I - S) (det R = 1) = (s2 + s3)(s1 + s3)(s1 + s2) over the
			// eigenvalues s of S = R^T F.
			if (!(fabs((sg[1] + sg[2]) * (sg[0] + sg[2]) * (sg[0] + sg[1])) > 1e-12)) flags |= 4;
		}
		else
			polar_svd(F, R);
		flags |= 1;
	}
	return flags;
}

// Derivative of the polar factor along a dual F: with R given (its value, row-major) and F = R S, S
// symmetric, R^T dF - dF^T R = [(tr(S) I - S) w]x for dR = R [w]x, so w solves a 3x3 system whose
// matrix is the element's G up to the rotation (zero derivative where that matrix is singular, where
// the tangent's rotation terms are dropped too).
template <typename S>
__host__ __device__ __forceinline__ void polar_tangent(const ad::DualT<S> (&F)[9], const S* Rv, ad::DualT<S> (&R)[9])
{
	S A[9], Sm[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			A[3 * i + j] = Rv[i] * F[j].d + Rv[3 + i] * F[3 + j].d + Rv[6 + i] * F[6 + j].d;  // R^T dF
			Sm[3 * i + j] = Rv[i] * F[j].v + Rv[3 + i] * F[3 + j].v + Rv[6 + i] * F[6 + j].v;  // R^T F
		}
	const S ax[3] = {A[7] - A[5], A[2] - A[6], A[3] - A[1]};  // axial(R^T dF - dF^T R)
	const S s01 = S(0.5) * (Sm[1] + Sm[3]), s02 = S(0.5) * (Sm[2] + Sm[6]), s12 = S(0.5) * (Sm[5] + Sm[7]);
	const S tr = Sm[0] + Sm[4] + Sm[8];
	const S M[9] = {tr - Sm[0], -s01, -s02, -s01, tr - Sm[4], -s12, -s02, -s12, tr - Sm[8]};
	S C[9];
	cofactor3(M, C);  // symmetric M: M^-1 = C / det
	const S det = M[0] * C[0] + M[1] * C[1] + M[2] * C[2];
	const S id = (fabs(det) > S(1e-12)) ? S(1) / det : S(0);
	const S w[3] = {(C[0] * ax[0] + C[1] * ax[1] + C[2] * ax[2]) * id, (C[3] * ax[0] + C[4] * ax[1] + C[5] * ax[2]) * id,
					(C[6] * ax[0] + C[7] * ax[1] + C[8] * ax[2]) * id};
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		const S* r = Rv + 3 * i;  // row i of R times [w]x
		const S d[3] = {r[1] * w[2] - r[2] * w[1], r[2] * w[0] - r[0] * w[2], r[0] * w[1] - r[1] * w[0]};
#pragma unroll
		for (int j = 0; j < 3; ++j) R[3 * i + j] = ad::DualT<S>::make(Rv[3 * i + j], d[j]);
	}
}

// Where compute_to() delivers an element's results. An output policy has
//   blocks()                    whether the stored lower-triangle blocks are wanted,
//   rhs_entry(j, v)             right-hand-side entry j = 3a+i,
//   block(a, b, slot, blk)      stored block (a, b) (a == b, or node a's id above node b's) in slot,
//   kAll, full_block(a, b, blk) when kAll, every one of the 16 blocks of the full tangent.
// StoreOut writes the stored blocks and the right-hand side to strided arrays (the forward kernels).
template <typename T>
struct StoreOut
{
	T* ks;
	int ksStride;
	T* rhs;
	int rhsStride;
	static constexpr bool kAll = false;
	__host__ __device__ __forceinline__ bool blocks() const { return ks != nullptr; }
	__host__ __device__ __forceinline__ void rhs_entry(int j, const T& v) { rhs[j * rhsStride] = v; }
	__host__ __device__ __forceinline__ void block(int, int, int slot, const T (&blk)[9])
	{
#pragma unroll
		for (int k = 0; k < 9; ++k) ks[(slot * 9 + k) * ksStride] = blk[k];
	}
	__host__ __device__ __forceinline__ void full_block(int, int, const T (&)[9]) {}
};

// Rotation, tangent blocks and right-hand-side share of one element, delivered to `out`:
//   the stored blocks: the element's lower-triangle blocks (kSlots of them);
//   the right-hand side, j = 3a+i: f_e + K_e uK + M0 uM (the element's share of the
//   implicit-Euler right-hand side, OdeSolverEulerImplicit.cpp:155-158, with the Rayleigh
//   damping force of FemRepresentation.cpp:565-629 folded in).
// Debug outputs (double only): kfull[144] the full tangent, fdbg[12] = f_e - alpha M0 v - beta K_e v.
// kLinear: the linear tetrahedron of Fem3DElementTetrahedron::doUpdateFMDK
// (Fem3DElementTetrahedron.cpp:77-90): R = I, K_e = K0, f_e = -K0 (x - x0), no rotation terms.
// The shape-function gradients g, the moduli and cm, and the inputs other than the positions are
// plain scalars G (for a dual T, its value type: only the positions carry a derivative).
// kGivenR: the rotation's value is Rgiven with the flags rflags of rotation(), as computed by a plain
// pass over the same element; a dual T takes its derivative from polar_tangent().
// Returns a bitmask: 1 = polar fallback to the FP64 SVD, 2 = singular G (extra terms skipped);
// 4 is internal (the FP32 form's FP64 singular-G decision on the SVD path).
template <typename T, bool kDebug, typename In, bool kLinear, typename Out, bool kGivenR = IsDual<T>::value>
__host__ __device__ int compute_to(const In& in, const typename ScalarOf<T>::type (&g)[4][3],
								   typename ScalarOf<T>::type lamV, typename ScalarOf<T>::type muV,
								   typename ScalarOf<T>::type cm, Out& out, double* kfull, double* fdbg,
								   const typename ScalarOf<T>::type* Rgiven = nullptr, int rflags = 0)
{
	static_assert(kGivenR || !IsDual<T>::value, "a dual pass takes the rotation's value from a plain pass");
	using G = typename ScalarOf<T>::type;
	int flags = 0;
	T F[9];
	deformation<T, kLinear>(in, g, F);
	T R[9];
	if constexpr (kGivenR)
	{
		flags = rflags;
		if constexpr (IsDual<T>::value)
			polar_tangent(F, Rgiven, R);
		else
		{
#pragma unroll
			for (int k = 0; k < 9; ++k) R[k] = Rgiven[k];
		}
	}
	else
		flags = rotation<T, kLinear>(in, g, F, R);
	// S = sym(R^T F), G = (tr(S) I - S) R^T (:208), G^-1 with the |det| > 1e-12 check (:210).
	T S[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) S[3 * i + j] = R[i] * F[j] + R[3 + i] * F[3 + j] + R[6 + i] * F[6 + j];
	{
		const T s01 = T(0.5) * (S[1] + S[3]), s02 = T(0.5) * (S[2] + S[6]), s12 = T(0.5) * (S[5] + S[7]);
		S[1] = S[3] = s01;
		S[2] = S[6] = s02;
		S[5] = S[7] = s12;
	}
	const T trS = S[0] + S[4] + S[8];
	T Gm[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			T s = 0;
#pragma unroll
			for (int k = 0; k < 3; ++k) s += ((i == k ? trS : T(0)) - S[3 * i + k]) * R[3 * j + k];
			Gm[3 * i + j] = s;
		}
	T Gi[9];
	bool extra = false;
	if constexpr (!kLinear)
	{
		T C[9];
		cofactor3(Gm, C);
		const T d = Gm[0] * C[0] + Gm[1] * C[1] + Gm[2] * C[2];
		// (An FP32 form of this test moved the FP32 element kernel from 168 to 190 registers, one
		// block per SM fewer; the conversion costs less than that.)
		extra = (std::is_same<G, float>::value && (flags & 1)) ? !(flags & 4) : fabs(double(d)) > 1e-12;
		const T id = T(1) / d;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) Gi[3 * i + j] = C[3 * j + i] * id;
		if (!extra) flags |= 2;
	}
	// Corotated strain displacement w_c = R^T p_c - q_c and u~_c = R^T uK_c - w_c.
	T w[4][3], ut[4][3], wt[4][3];
	if constexpr (kLinear)
	{
		// u = x - x0 relative to node 0 (K0 annihilates translations), formed in the input precision.
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				w[a][i] = T(in.p[a][i] - in.q[a][i]);
				ut[a][i] = T(in.uK[a][i]) - w[a][i];
			}
	}
	else if constexpr (!std::is_same<T, float>::value)
	{
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				w[a][i] = R[i] * T(in.p[a][0]) + R[3 + i] * T(in.p[a][1]) + R[6 + i] * T(in.p[a][2]) - G(in.q[a][i]);
				ut[a][i] = R[i] * G(in.uK[a][0]) + R[3 + i] * G(in.uK[a][1]) + R[6 + i] * G(in.uK[a][2]) - w[a][i];
			}
	}
	else
	{
		// An FP32 rotation is orthogonal only to ~1e-7, and its symmetric error would read as a
		// spurious strain of that size. Since p_a = F q_a and F = R S, R^T p_a - q_a = (S - I) q_a,
		// with S - I = (C - I)(S + I)^-1 and C - I = sum_ab (p_a.p_b - q_a.q_b) g_a g_b^T: the Gram
		// differences are formed without loss to cancellation (gram_diff), everything after in FP32
		// with eps32-relative accuracy.
		T Dl[3][3];
#pragma unroll
		for (int a = 0; a < 3; ++a)
#pragma unroll
			for (int c = a; c < 3; ++c) Dl[a][c] = Dl[c][a] = gram_diff(in, a + 1, c + 1);
		T CD[3][3], CmI[9];  // CD = Dl G^T (rows a), CmI = G Dl G^T with G = [g_1 g_2 g_3]
#pragma unroll
		for (int a = 0; a < 3; ++a)
#pragma unroll
			for (int j = 0; j < 3; ++j) CD[a][j] = T(Dl[a][0]) * g[1][j] + T(Dl[a][1]) * g[2][j] + T(Dl[a][2]) * g[3][j];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) CmI[3 * i + j] = g[1][i] * CD[0][j] + g[2][i] * CD[1][j] + g[3][i] * CD[2][j];
		T SpI[9], C[9], Em[9];
#pragma unroll
		for (int k = 0; k < 9; ++k) SpI[k] = S[k] + ((k % 4 == 0) ? T(1) : T(0));
		cofactor3(SpI, C);
		const T idet = T(1) / (SpI[0] * C[0] + SpI[1] * C[1] + SpI[2] * C[2]);
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)  // (C - I) (S + I)^-1, inverse = cofactor^T / det
				Em[3 * i + j] = (CmI[3 * i] * C[3 * j] + CmI[3 * i + 1] * C[3 * j + 1] + CmI[3 * i + 2] * C[3 * j + 2]) * idet;
		const T e01 = T(0.5) * (Em[1] + Em[3]), e02 = T(0.5) * (Em[2] + Em[6]), e12 = T(0.5) * (Em[5] + Em[7]);
		Em[1] = Em[3] = e01;
		Em[2] = Em[6] = e02;
		Em[5] = Em[7] = e12;
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				w[a][i] = Em[3 * i] * rest_edge(in, a, 0) + Em[3 * i + 1] * rest_edge(in, a, 1) + Em[3 * i + 2] * rest_edge(in, a, 2);
				ut[a][i] = R[i] * G(in.uK[a][0]) + R[3 + i] * G(in.uK[a][1]) + R[6 + i] * G(in.uK[a][2]) - w[a][i];
			}
	}
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i) wt[a][i] = R[i] * w[a][0] + R[3 + i] * w[a][1] + R[6 + i] * w[a][2];  // R^T w
	G Gab[4][4];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int c = 0; c < 4; ++c) Gab[a][c] = g[a][0] * g[c][0] + g[a][1] * g[c][1] + g[a][2] * g[c][2];
	T h[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i) h[a][i] = R[3 * i] * g[a][0] + R[3 * i + 1] * g[a][1] + R[3 * i + 2] * g[a][2];
	// y = Krot w = R K0 (R^T w) (KTimesRx_x0); Ry_a = R y_a.
	T tmp[4][3], Ry[4][3];
	k0_apply(g, Gab, lamV, muV, wt, tmp);
#pragma unroll
	for (int a = 0; a < 4; ++a)
	{
		T ya[3];
#pragma unroll
		for (int i = 0; i < 3; ++i) ya[i] = R[3 * i] * tmp[a][0] + R[3 * i + 1] * tmp[a][1] + R[3 * i + 2] * tmp[a][2];
#pragma unroll
		for (int i = 0; i < 3; ++i) Ry[a][i] = R[3 * i] * ya[0] + R[3 * i + 1] * ya[1] + R[3 * i + 2] * ya[2];
	}
	// zeta = sum_c g_c x w_c, W[i] = sum_c g_c[i] w_c, zt = sum_c g_c x u~_c.
	T zeta[3] = {0, 0, 0}, zt[3] = {0, 0, 0}, W[3][3];
#pragma unroll
	for (int c = 0; c < 4; ++c)
	{
		T cr[3];
		cross3(g[c], w[c], cr);
		zeta[0] += cr[0];
		zeta[1] += cr[1];
		zeta[2] += cr[2];
		cross3(g[c], ut[c], cr);
		zt[0] += cr[0];
		zt[1] += cr[1];
		zt[2] += cr[2];
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) W[i][j] = g[0][i] * w[0][j] + g[1][i] * w[1][j] + g[2][i] * w[2][j] + g[3][i] * w[3][j];
	// g_b x r_q for every node b and row q of R: held for the whole node loop, or (dual passes, whose
	// per-thread state is what bounds them) formed again for each block.
	constexpr bool kLean = IsDual<T>::value;
	T cbq[kLean ? 1 : 4][3][3];
	if constexpr (!kLean)
	{
#pragma unroll
		for (int bb = 0; bb < 4; ++bb)
#pragma unroll
			for (int qq = 0; qq < 3; ++qq) cross3(g[bb], &R[3 * qq], cbq[bb][qq]);
	}
	T Ku[4][3];
	k0_apply(g, Gab, lamV, muV, ut, Ku);
	T KW[4][3];
	if (kDebug) k0_apply(g, Gab, lamV, muV, w, KW);
	G sumM[3], sumV[3];
#pragma unroll
	for (int k = 0; k < 3; ++k)
	{
		sumM[k] = G(in.uM[0][k] + in.uM[1][k] + in.uM[2][k] + in.uM[3][k]);
		sumV[k] = G(in.vv[0][k] + in.vv[1][k] + in.vv[2][k] + in.vv[3][k]);
	}

#pragma unroll
	for (int a = 0; a < 4; ++a)
	{
		// L_a = lambdaV g_a zeta^T + muV [rows: g_a x W_i] + muV [sum_c G_ac w_c]x   (local frame)
		T L[9], sw[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) sw[k] = Gab[a][0] * w[0][k] + Gab[a][1] * w[1][k] + Gab[a][2] * w[2][k] + Gab[a][3] * w[3][k];
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			T cr[3];
			cross3(g[a], W[i], cr);
#pragma unroll
			for (int j = 0; j < 3; ++j) L[3 * i + j] = lamV * g[a][i] * zeta[j] + muV * cr[j];
		}
		L[1] -= muV * sw[2];
		L[2] += muV * sw[1];
		L[3] += muV * sw[2];
		L[5] -= muV * sw[0];
		L[6] -= muV * sw[1];
		L[7] += muV * sw[0];
		// T_a = -[R y_a]x + R L R^T ; T'_a = T_a G^-1
		T RL[9], Tm[9], Tp[9];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) RL[3 * i + j] = R[3 * i] * L[j] + R[3 * i + 1] * L[3 + j] + R[3 * i + 2] * L[6 + j];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
				Tm[3 * i + j] = RL[3 * i] * R[3 * j] + RL[3 * i + 1] * R[3 * j + 1] + RL[3 * i + 2] * R[3 * j + 2];
		Tm[1] += Ry[a][2];
		Tm[2] -= Ry[a][1];
		Tm[3] -= Ry[a][2];
		Tm[5] += Ry[a][0];
		Tm[6] += Ry[a][1];
		Tm[7] -= Ry[a][0];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
				Tp[3 * i + j] = extra ? (Tm[3 * i] * Gi[j] + Tm[3 * i + 1] * Gi[3 + j] + Tm[3 * i + 2] * Gi[6 + j]) : T(0);

		// rhs_a = R K0(u~)_a + T'_a zt + (M0 uM)_a, M0 uM = cm (uM_a + sum uM); with mass lumping
		// (FemRepresentation.cpp:499-508) each row of M0 is summed onto its diagonal, 5 cm = rho V / 4.
#pragma unroll
		for (int i = 0; i < 3; ++i)
			out.rhs_entry(3 * a + i, R[3 * i] * Ku[a][0] + R[3 * i + 1] * Ku[a][1] + R[3 * i + 2] * Ku[a][2] +
										 Tp[3 * i] * zt[0] + Tp[3 * i + 1] * zt[1] + Tp[3 * i + 2] * zt[2] +
										 (in.lumped ? cm * G(5) * G(in.uM[a][i]) : cm * (G(in.uM[a][i]) + sumM[i])));

		T kv[3] = {0, 0, 0};
#pragma unroll
		for (int bb = 0; bb < 4; ++bb)
		{
			const bool store = ((a == bb) || (in.nd[a] > in.nd[bb])) && out.blocks();
			if (!store && !kDebug && !Out::kAll) continue;
			T cb[3][3];
#pragma unroll
			for (int qq = 0; qq < 3; ++qq)
			{
				if constexpr (kLean)
					cross3(g[bb], &R[3 * qq], cb[qq]);
				else
				{
#pragma unroll
					for (int k = 0; k < 3; ++k) cb[qq][k] = cbq[bb][qq][k];
				}
			}
			T blk[9];
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int qq = 0; qq < 3; ++qq)
				{
					T v = lamV * h[a][i] * h[bb][qq] + muV * h[bb][i] * h[a][qq] + Tp[3 * i] * cb[qq][0] +
						  Tp[3 * i + 1] * cb[qq][1] + Tp[3 * i + 2] * cb[qq][2];
					if (i == qq) v = v + muV * Gab[a][bb];
					blk[3 * i + qq] = v;
				}
			if (store) out.block(a, bb, (a == bb) ? a : pair_slot(a < bb ? a : bb, a < bb ? bb : a), blk);
			if (Out::kAll) out.full_block(a, bb, blk);
			if (kDebug)
			{
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
#pragma unroll
					for (int qq = 0; qq < 3; ++qq) kfull[(3 * a + i) * 12 + 3 * bb + qq] = double(blk[3 * i + qq]);
					kv[i] += blk[3 * i] * G(in.vv[bb][0]) + blk[3 * i + 1] * G(in.vv[bb][1]) + blk[3 * i + 2] * G(in.vv[bb][2]);
				}
			}
		}
		if (kDebug)
		{
			// f_e - alpha M0 v - beta K_e v, with f_e = -(R K0(w)_a + T'_a zeta)  (:103-113).
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				const T fe = -(R[3 * i] * KW[a][0] + R[3 * i + 1] * KW[a][1] + R[3 * i + 2] * KW[a][2] +
							   Tp[3 * i] * zeta[0] + Tp[3 * i + 1] * zeta[1] + Tp[3 * i + 2] * zeta[2]);
				const G mv = in.lumped ? cm * G(5) * G(in.vv[a][i]) : cm * (G(in.vv[a][i]) + sumV[i]);
				fdbg[3 * a + i] = double(fe) - in.alphaDbg * double(mv) - in.betaDbg * double(kv[i]);
			}
		}
	}
	return flags;
}

// compute_to() with the results written to strided arrays: ks[k * ksStride], k = slot*9 + entry,
// the stored blocks (ks may be null: right-hand side only); rhs[j * rhsStride], j = 3a+i.
template <typename T, bool kDebug, typename In = ElemIn, bool kLinear = false>
__host__ __device__ __forceinline__ int compute(const In& in, const T (&g)[4][3], T lamV, T muV, T cm, T* ks,
												int ksStride, T* rhs, int rhsStride, double* kfull, double* fdbg)
{
	StoreOut<T> out{ks, ksStride, rhs, rhsStride};
	return compute_to<T, kDebug, In, kLinear>(in, g, lamV, muV, cm, out, kfull, fdbg);
}

}  // namespace elem
}  // namespace gbfem
