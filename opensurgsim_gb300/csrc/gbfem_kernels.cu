// gbfem_kernels.cu -- sm_103a kernels of the corotational-tetrahedron implicit-Euler step.
//
// Element kernel (one element per thread): deformation gradient, polar decomposition, the
// corotational tangent stiffness (R K0 R^T plus the dR/dx terms of
// Fem3DElementCorotationalTetrahedron.cpp:199-286, including the reference's use of the rotated
// stiffness in KTimesRx_x0, :276) and the element's share of the implicit-Euler right-hand side.
// Assembly gathers element blocks through a precomputed map (deterministic, element order), the
// right-hand side gathers per node, and the Jacobi-preconditioned CG reads the symmetric matrix
// built from the lower triangle, as Eigen's ConjugateGradient<..., Lower> does.
//
// The element math is written in closed form on the shape-function gradients g_a instead of
// 12x12 products: with h_a = R g_a and G_ab = g_a . g_b,
//   K0_ab   = V (lambda g_a g_b^T + mu g_b g_a^T + mu G_ab I)            (= V B^T Em B)
//   Krot_ab = V (lambda h_a h_b^T + mu h_b h_a^T + mu G_ab I)            (= R K0_ab R^T)
//   dR/dx_(b,q) = [psi_bq]x R,  psi_bq = G^-1 (g_b x r_q),  r_q = row q of R
//   extra(3a+i, 3b+q) = (T_a G^-1 (g_b x r_q))_i,
//   T_a = -[R y_a]x + R (sum_c K0_ac [w_c]x) R^T,  w_c = R^T (x_c - x_0) - (x0_c - x0_0),
//   y = Krot w  (the reference's KTimesRx_x0).
// All quantities are formed on positions relative to node 0, which the tangent annihilates.

#include <cfloat>
#include <cstdint>

#include "gbfem_internal.h"

namespace gbfem {

namespace {

constexpr int kVecThreads = 256;

// ------------------------------------------------------------------------------------------
// Small 3x3 helpers (row-major arrays of 9).
// ------------------------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ void cofactor3(const T* X, T* C)
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
__device__ __forceinline__ T det3(const T* X)
{
	return X[0] * (X[4] * X[8] - X[5] * X[7]) - X[1] * (X[3] * X[8] - X[5] * X[6]) + X[2] * (X[3] * X[7] - X[4] * X[6]);
}

template <typename T>
__device__ __forceinline__ void cross3(const T* a, const T* b, T* c)
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
	static constexpr double newtonTol2 = 1e-26;  // |X_k+1 - X_k|_F^2
};
template <>
struct Eps<float>
{
	static constexpr float eps = FLT_EPSILON;
	static constexpr float newtonTol2 = 1e-11f;
};

// Polar factor by Newton's iteration X <- (g X + X^-T / g) / 2 (Higham), Frobenius scaling on
// the first iterations. Valid for det F > 0, where the rotation equals the SVD-based result of
// Transform::computeRotationScaling. Returns false (caller falls back to the SVD) otherwise or
// when the iteration does not settle within the bound.
template <typename T>
__device__ bool polar_newton(const T* F, T* R)
{
	T X[9];
#pragma unroll
	for (int k = 0; k < 9; ++k) X[k] = F[k];
	for (int it = 0; it < 20; ++it)
	{
		T C[9];
		cofactor3(X, C);
		T d = X[0] * C[0] + X[1] * C[1] + X[2] * C[2];
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
			gam = sqrt(sqrt(nc / (nx * d * d)));
		}
		T a = T(0.5) * gam;
		T b = T(0.5) / (gam * d);
		T diff = 0;
#pragma unroll
		for (int k = 0; k < 9; ++k)
		{
			T xn = a * X[k] + b * C[k];
			T dd = xn - X[k];
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

// SVD-based polar factor for any F (one-sided Jacobi, bounded sweeps), proper rotation with the
// reflection placed on the smallest singular value.
template <typename T>
__device__ void polar_svd(const T* F, T* R)
{
	T A[9], V[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
#pragma unroll
	for (int k = 0; k < 9; ++k) A[k] = F[k];
	for (int sweep = 0; sweep < 40; ++sweep)
	{
		bool rotated = false;
		for (int pp = 0; pp < 3; ++pp)
		{
			int p = (pp == 2) ? 1 : 0;
			int q = (pp == 0) ? 1 : 2;
			T al = 0, be = 0, ga = 0;
			for (int k = 0; k < 3; ++k)
			{
				al += A[3 * k + p] * A[3 * k + p];
				be += A[3 * k + q] * A[3 * k + q];
				ga += A[3 * k + p] * A[3 * k + q];
			}
			if (ga == T(0) || fabs(ga) <= Eps<T>::eps * sqrt(al * be)) continue;
			rotated = true;
			T zeta = (be - al) / (T(2) * ga);
			T t = (zeta >= T(0) ? T(1) : T(-1)) / (fabs(zeta) + sqrt(T(1) + zeta * zeta));
			T c = T(1) / sqrt(T(1) + t * t);
			T s = c * t;
			for (int k = 0; k < 3; ++k)
			{
				T ap = A[3 * k + p], aq = A[3 * k + q];
				A[3 * k + p] = c * ap - s * aq;
				A[3 * k + q] = s * ap + c * aq;
				T vp = V[3 * k + p], vq = V[3 * k + q];
				V[3 * k + p] = c * vp - s * vq;
				V[3 * k + q] = s * vp + c * vq;
			}
		}
		if (!rotated) break;
	}
	T sv[3];
	for (int j = 0; j < 3; ++j) sv[j] = sqrt(A[j] * A[j] + A[3 + j] * A[3 + j] + A[6 + j] * A[6 + j]);
	int o[3] = {0, 1, 2};
	if (sv[o[0]] < sv[o[1]]) { int tt = o[0]; o[0] = o[1]; o[1] = tt; }
	if (sv[o[1]] < sv[o[2]]) { int tt = o[1]; o[1] = o[2]; o[2] = tt; }
	if (sv[o[0]] < sv[o[1]]) { int tt = o[0]; o[0] = o[1]; o[1] = tt; }
	T U[9], Vs[9];
	for (int j = 0; j < 3; ++j)
		for (int k = 0; k < 3; ++k) Vs[3 * k + j] = V[3 * k + o[j]];
	T smax = sv[o[0]] > T(0) ? sv[o[0]] : T(1);
	for (int j = 0; j < 3; ++j)
	{
		T s = sv[o[j]];
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
			// Rank < 2: complete with the canonical axis least aligned with column 0, orthonormalised.
			int ax = 0;
			T best = T(2);
			for (int a = 0; a < 3; ++a)
			{
				T d = (j == 0) ? T(0) : fabs(U[3 * a]);
				if (d < best) { best = d; ax = a; }
			}
			T e[3] = {T(ax == 0), T(ax == 1), T(ax == 2)};
			if (j == 1)
			{
				T d = e[0] * U[0] + e[1] * U[3] + e[2] * U[6];
				for (int k = 0; k < 3; ++k) e[k] -= d * U[3 * k];
			}
			T nrm = sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
			for (int k = 0; k < 3; ++k) U[3 * k + j] = e[k] / nrm;
		}
	}
	T x = (det3(U) * det3(Vs) < T(0)) ? T(-1) : T(1);
	for (int k = 0; k < 3; ++k) U[3 * k + 2] *= x;
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) R[3 * i + j] = U[3 * i] * Vs[3 * j] + U[3 * i + 1] * Vs[3 * j + 1] + U[3 * i + 2] * Vs[3 * j + 2];
}

// (K0 u)_a = lambdaV tr(D) g_a + muV D^T g_a + muV sum_c G_ac u_c,  D = sum_c u_c g_c^T.
template <typename T>
__device__ __forceinline__ void k0_apply(const T (&g)[4][3], const T (&Gab)[4][4], T lamV, T muV, const T (&u)[4][3],
										 T (&out)[4][3])
{
	T D[3][3];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) D[i][j] = u[0][i] * g[0][j] + u[1][i] * g[1][j] + u[2][i] * g[2][j] + u[3][i] * g[3][j];
	T tr = D[0][0] + D[1][1] + D[2][2];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int j = 0; j < 3; ++j)
			out[a][j] = lamV * tr * g[a][j] + muV * (D[0][j] * g[a][0] + D[1][j] * g[a][1] + D[2][j] * g[a][2]) +
						muV * (Gab[a][0] * u[0][j] + Gab[a][1] * u[1][j] + Gab[a][2] * u[2][j] + Gab[a][3] * u[3][j]);
}

__device__ __forceinline__ int pair_slot(int a, int b)
{
	// (0,1)->4 (0,2)->5 (0,3)->6 (1,2)->7 (1,3)->8 (2,3)->9 for a < b
	return (a == 0) ? (3 + b) : (a == 1 ? (5 + b) : 9);
}

// ------------------------------------------------------------------------------------------
// Element kernel, FP64. One element per thread.
// ------------------------------------------------------------------------------------------
template <bool kDebug>
__global__ void __launch_bounds__(64) k_element_fp64(DevBody b, const double* __restrict__ xn,
													  const double* __restrict__ vn, const double* __restrict__ xt,
													  const double* __restrict__ vt, double dt, double alpha,
													  double beta, double* __restrict__ kslots,
													  double* __restrict__ rhsE, double* __restrict__ kfull,
													  double* __restrict__ fE, int* counters)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= b.E) return;
	const int E = b.E;
	const int4 t4 = b.tets[e];
	const int nd[4] = {t4.x, t4.y, t4.z, t4.w};
	double g[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k) g[a][k] = b.rest[(3 * a + k) * E + e];
	const double lamV = b.rest[13 * E + e], muV = b.rest[14 * E + e], cm = b.rest[15 * E + e];

	// Relative positions (node 0 is the origin) and the right-hand-side operands per node:
	//   uK = -beta v_n + (x_n - x_t - dt v_n),  uM = -alpha v_n - (v_n - v_t)/dt.
	double p[4][3], q[4][3], uK[4][3], uM[4][3], vv[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			const int d = 3 * nd[a] + k;
			const double xa = xn[d], va = vn[d];
			p[a][k] = xa - xn[3 * nd[0] + k];
			q[a][k] = b.xrest[d] - b.xrest[3 * nd[0] + k];
			uK[a][k] = -beta * va + ((xa - xt[d]) - dt * va);
			uM[a][k] = -alpha * va - (va - vt[d]) / dt;
			vv[a][k] = va;
		}
	// F = sum_a p_a g_a^T (linear part of P V^-1, Fem3DElementCorotationalTetrahedron.cpp:146).
	double F[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) F[3 * i + j] = p[1][i] * g[1][j] + p[2][i] * g[2][j] + p[3][i] * g[3][j];
	double R[9];
	if (!polar_newton(F, R))
	{
		polar_svd(F, R);
		atomicAdd(&counters[1], 1);
	}
	// S = R^T F (symmetric part), G = (tr(S) I - S) R^T (:208).
	double S[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j) S[3 * i + j] = R[i] * F[j] + R[3 + i] * F[3 + j] + R[6 + i] * F[6 + j];
	{
		double s01 = 0.5 * (S[1] + S[3]), s02 = 0.5 * (S[2] + S[6]), s12 = 0.5 * (S[5] + S[7]);
		S[1] = S[3] = s01;
		S[2] = S[6] = s02;
		S[5] = S[7] = s12;
	}
	const double trS = S[0] + S[4] + S[8];
	double Gm[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			double s = 0;
#pragma unroll
			for (int k = 0; k < 3; ++k) s += ((i == k ? trS : 0.0) - S[3 * i + k]) * R[3 * j + k];
			Gm[3 * i + j] = s;
		}
	double Gi[9];
	bool extra;
	{
		double C[9];
		cofactor3(Gm, C);
		const double d = Gm[0] * C[0] + Gm[1] * C[1] + Gm[2] * C[2];
		extra = fabs(d) > 1e-12;  // computeInverseAndDetWithCheck threshold (:210)
		const double id = 1.0 / d;
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) Gi[3 * i + j] = C[3 * j + i] * id;
		if (!extra) atomicAdd(&counters[0], 1);
	}
	// w_c = R^T p_c - q_c (local frame), u~_c = R^T uK_c - w_c.
	double w[4][3], ut[4][3], wt[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			w[a][i] = R[i] * p[a][0] + R[3 + i] * p[a][1] + R[6 + i] * p[a][2] - q[a][i];
			ut[a][i] = R[i] * uK[a][0] + R[3 + i] * uK[a][1] + R[6 + i] * uK[a][2];
		}
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			ut[a][i] -= w[a][i];
			wt[a][i] = R[i] * w[a][0] + R[3 + i] * w[a][1] + R[6 + i] * w[a][2];  // R^T w
		}
	double Gab[4][4];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int c = 0; c < 4; ++c) Gab[a][c] = g[a][0] * g[c][0] + g[a][1] * g[c][1] + g[a][2] * g[c][2];
	double h[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i) h[a][i] = R[3 * i] * g[a][0] + R[3 * i + 1] * g[a][1] + R[3 * i + 2] * g[a][2];

	// y = Krot w = R K0 (R^T w)  (KTimesRx_x0, :276); Ry_a = R y_a.
	double tmp[4][3], Ry[4][3];
	k0_apply(g, Gab, lamV, muV, wt, tmp);
#pragma unroll
	for (int a = 0; a < 4; ++a)
	{
		double ya[3];
#pragma unroll
		for (int i = 0; i < 3; ++i) ya[i] = R[3 * i] * tmp[a][0] + R[3 * i + 1] * tmp[a][1] + R[3 * i + 2] * tmp[a][2];
#pragma unroll
		for (int i = 0; i < 3; ++i) Ry[a][i] = R[3 * i] * ya[0] + R[3 * i + 1] * ya[1] + R[3 * i + 2] * ya[2];
	}
	// zeta = sum_c g_c x w_c, W[i] = sum_c g_c[i] w_c, zt = sum_c g_c x u~_c.
	double zeta[3] = {0, 0, 0}, zt[3] = {0, 0, 0}, W[3][3];
#pragma unroll
	for (int c = 0; c < 4; ++c)
	{
		double cr[3];
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
	// c_bq = g_b x r_q.
	double cbq[4][3][3];
#pragma unroll
	for (int bb = 0; bb < 4; ++bb)
#pragma unroll
		for (int qq = 0; qq < 3; ++qq) cross3(g[bb], &R[3 * qq], cbq[bb][qq]);
	// Right-hand side: rhs_a = R K0(u~)_a + T'_a zt + cm (uM_a + sum uM).
	double Ku[4][3];
	k0_apply(g, Gab, lamV, muV, ut, Ku);
	double KW[4][3];
	if (kDebug) k0_apply(g, Gab, lamV, muV, w, KW);
	double sumM[3] = {uM[0][0] + uM[1][0] + uM[2][0] + uM[3][0], uM[0][1] + uM[1][1] + uM[2][1] + uM[3][1],
					  uM[0][2] + uM[1][2] + uM[2][2] + uM[3][2]};
	double sumV[3] = {vv[0][0] + vv[1][0] + vv[2][0] + vv[3][0], vv[0][1] + vv[1][1] + vv[2][1] + vv[3][1],
					  vv[0][2] + vv[1][2] + vv[2][2] + vv[3][2]};
	double* ks = kslots + (size_t)e * (kSlots * 9);

#pragma unroll 1
	for (int a = 0; a < 4; ++a)
	{
		// L_a = lambdaV g_a zeta^T + muV [rows: g_a x W_i] + muV [sum_c G_ac w_c]x   (local frame)
		double L[9];
		double sw[3];
#pragma unroll
		for (int k = 0; k < 3; ++k) sw[k] = Gab[a][0] * w[0][k] + Gab[a][1] * w[1][k] + Gab[a][2] * w[2][k] + Gab[a][3] * w[3][k];
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			double cr[3];
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
		double RL[9], T[9];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) RL[3 * i + j] = R[3 * i] * L[j] + R[3 * i + 1] * L[3 + j] + R[3 * i + 2] * L[6 + j];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) T[3 * i + j] = RL[3 * i] * R[3 * j] + RL[3 * i + 1] * R[3 * j + 1] + RL[3 * i + 2] * R[3 * j + 2];
		T[1] += Ry[a][2];
		T[2] -= Ry[a][1];
		T[3] -= Ry[a][2];
		T[5] += Ry[a][0];
		T[6] += Ry[a][1];
		T[7] -= Ry[a][0];
		double Tp[9];
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
				Tp[3 * i + j] = extra ? (T[3 * i] * Gi[j] + T[3 * i + 1] * Gi[3 + j] + T[3 * i + 2] * Gi[6 + j]) : 0.0;

		// rhs block a
		double ra[3];
#pragma unroll
		for (int i = 0; i < 3; ++i)
			ra[i] = R[3 * i] * Ku[a][0] + R[3 * i + 1] * Ku[a][1] + R[3 * i + 2] * Ku[a][2] + Tp[3 * i] * zt[0] +
					Tp[3 * i + 1] * zt[1] + Tp[3 * i + 2] * zt[2] + cm * (uM[a][i] + sumM[i]);
#pragma unroll
		for (int i = 0; i < 3; ++i) rhsE[(size_t)e * 12 + 3 * a + i] = ra[i];

		double kv[3] = {0, 0, 0};
#pragma unroll 1
		for (int bb = 0; bb < 4; ++bb)
		{
			const bool store = (a == bb) || (nd[a] > nd[bb]);
			if (!store && !kDebug) continue;
			double blk[9];
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int qq = 0; qq < 3; ++qq)
				{
					double v = lamV * h[a][i] * h[bb][qq] + muV * h[bb][i] * h[a][qq] +
							   Tp[3 * i] * cbq[bb][qq][0] + Tp[3 * i + 1] * cbq[bb][qq][1] + Tp[3 * i + 2] * cbq[bb][qq][2];
					if (i == qq) v += muV * Gab[a][bb];
					blk[3 * i + qq] = v;
				}
			if (store)
			{
				const int slot = (a == bb) ? a : pair_slot(a < bb ? a : bb, a < bb ? bb : a);
#pragma unroll
				for (int k = 0; k < 9; ++k) ks[slot * 9 + k] = blk[k];
			}
			if (kDebug)
			{
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
#pragma unroll
					for (int qq = 0; qq < 3; ++qq) kfull[(size_t)e * 144 + (3 * a + i) * 12 + 3 * bb + qq] = blk[3 * i + qq];
					kv[i] += blk[3 * i] * vv[bb][0] + blk[3 * i + 1] * vv[bb][1] + blk[3 * i + 2] * vv[bb][2];
				}
			}
		}
		if (kDebug)
		{
			// f_e - alpha M0 v - beta K_e v, with f_e = -(R K0(w)_a + T'_a zeta)  (:103-113).
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				double fe = -(R[3 * i] * KW[a][0] + R[3 * i + 1] * KW[a][1] + R[3 * i + 2] * KW[a][2] +
							  Tp[3 * i] * zeta[0] + Tp[3 * i + 1] * zeta[1] + Tp[3 * i + 2] * zeta[2]);
				fE[(size_t)e * 12 + 3 * a + i] = fe - alpha * (cm * (vv[a][i] + sumV[i])) - beta * kv[i];
			}
		}
	}
}

// ------------------------------------------------------------------------------------------
// Assembly: one thread per lower block (I >= J). Sums element blocks in element order, forms
// S = c1 M + c2 K (c1 = 1/dt + alpha, c2 = dt + beta), applies boundary conditions
// (OdeState.cpp:197-218: zero rows and columns, diagonal 1) and writes the symmetric BSR matrix
// that Eigen's selfadjointView<Lower> implies.
// ------------------------------------------------------------------------------------------
__global__ void k_assemble_bsr(DevBody b, const double* __restrict__ ks, double c1, double c2, double* __restrict__ A,
							   double* __restrict__ invdiag)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	const int k1 = b.cptr[L + 1];
	for (int k = b.cptr[L]; k < k1; ++k)
	{
		const double* src = ks + (size_t)b.cidx[k] * 9;
#pragma unroll
		for (int m = 0; m < 9; ++m) s[m] += src[m];
	}
	const double mm = c1 * b.lmass[L];
	double blk[9];
#pragma unroll
	for (int m = 0; m < 9; ++m) blk[m] = c2 * s[m];
	blk[0] += mm;
	blk[4] += mm;
	blk[8] += mm;
	const int I = lb.x, J = lb.y;
	if (I == J)
	{
		blk[1] = blk[3];
		blk[2] = blk[6];
		blk[5] = blk[7];
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const int r = 3 * I + i, c = 3 * J + j;
			if (b.bc[r] | b.bc[c]) blk[3 * i + j] = (r == c) ? 1.0 : 0.0;
		}
#pragma unroll
	for (int m = 0; m < 9; ++m) A[(size_t)lb.z + 32 * m] = blk[m];
	if (lb.w >= 0)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) A[(size_t)lb.w + 32 * (3 * j + i)] = blk[3 * i + j];
	}
	if (I == J)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			const double d = blk[4 * i];
			invdiag[3 * I + i] = (d != 0.0) ? 1.0 / d : 1.0;  // DiagonalPreconditioner
		}
	}
}

__global__ void k_rhs_gather(DevBody b, const double* __restrict__ rhsE, double g0, double g1, double g2, int gravityOn,
							 double* __restrict__ rhs, int applyBc)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= b.N) return;
	double s0 = 0, s1 = 0, s2 = 0;
	const int k1 = b.iptr[I + 1];
	for (int k = b.iptr[I]; k < k1; ++k)
	{
		const int c = b.iidx[k];
		const double* src = rhsE + (size_t)(c >> 2) * 12 + 3 * (c & 3);
		s0 += src[0];
		s1 += src[1];
		s2 += src[2];
	}
	if (gravityOn)  // FemRepresentation::addGravityForce (:641-662)
	{
		const double m = b.nmass[I];
		s0 += g0 * m;
		s1 += g1 * m;
		s2 += g2 * m;
	}
	if (applyBc)
	{
		if (b.bc[3 * I]) s0 = 0.0;
		if (b.bc[3 * I + 1]) s1 = 0.0;
		if (b.bc[3 * I + 2]) s2 = 0.0;
	}
	rhs[3 * I] = s0;
	rhs[3 * I + 1] = s1;
	rhs[3 * I + 2] = s2;
}

__global__ void k_assemble_full_csc(int nnz, const int* __restrict__ sptr, const int* __restrict__ sidx,
									const int* __restrict__ srow, const int* __restrict__ scol,
									const double* __restrict__ kfull, const double* __restrict__ smass,
									const uint8_t* __restrict__ bc, double c1, double c2, double* __restrict__ S)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nnz) return;
	double s = 0;
	for (int t = sptr[k]; t < sptr[k + 1]; ++t) s += kfull[sidx[t]];
	double v = c1 * smass[k] + c2 * s;
	const int r = srow[k], c = scol[k];
	if (bc[r] | bc[c]) v = (r == c) ? 1.0 : 0.0;
	S[k] = v;
}

// ------------------------------------------------------------------------------------------
// Deterministic grid reductions: every block writes its partials, the last block to finish
// (ticket counter) sums them in block order. Results do not depend on scheduling.
// ------------------------------------------------------------------------------------------
struct OpSum
{
	__device__ static double apply(double a, double b) { return a + b; }
	__device__ static double identity() { return 0.0; }
};
struct OpMax
{
	__device__ static double apply(double a, double b) { return fmax(a, b); }
	__device__ static double identity() { return 0.0; }
};

template <typename Op>
__device__ __forceinline__ double warp_reduce(double v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = Op::apply(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

template <typename Op, int NV>
__device__ __forceinline__ void block_reduce(double (&v)[NV])
{
	__shared__ double sh[NV][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for (int k = 0; k < NV; ++k) v[k] = warp_reduce<Op>(v[k]);
	__syncthreads();
	if (lane == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k) sh[k][warp] = v[k];
	__syncthreads();
#pragma unroll
	for (int k = 0; k < NV; ++k)
	{
		double x = (lane < nw) ? sh[k][lane] : Op::identity();
		v[k] = warp_reduce<Op>(x);  // every warp holds the block total
	}
}

// Returns true in every thread of the last block, with tot[] = grid totals.
template <typename Op, int NV>
__device__ bool grid_reduce(double (&v)[NV], double* part, unsigned int* ticket, double (&tot)[NV])
{
	__shared__ bool amLast;
	block_reduce<Op, NV>(v);
	if (threadIdx.x == 0)
	{
#pragma unroll
		for (int k = 0; k < NV; ++k) part[k * gridDim.x + blockIdx.x] = v[k];
		__threadfence();
		const unsigned int t = atomicAdd(ticket, 1u);
		amLast = (t == gridDim.x - 1);
	}
	__syncthreads();
	if (!amLast) return false;
	__threadfence();
#pragma unroll
	for (int k = 0; k < NV; ++k)
	{
		double s = Op::identity();
		for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s = Op::apply(s, __ldcg(&part[k * gridDim.x + i]));
		tot[k] = s;
	}
	block_reduce<Op, NV>(tot);
	if (threadIdx.x == 0) *ticket = 0u;
	return true;
}

// ------------------------------------------------------------------------------------------
// Conjugate gradient (Eigen's conjugate_gradient with a Jacobi preconditioner, x0 = 0).
// ------------------------------------------------------------------------------------------
__global__ void k_cg_init(int n, const double* __restrict__ bvec, const double* __restrict__ invdiag,
						  double* __restrict__ x, double* __restrict__ r, double* __restrict__ p, CgCtl* ctl,
						  double* part, double tol, int maxIter)
{
	double v[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double bi = bvec[i];
		const double zi = invdiag[i] * bi;
		x[i] = 0.0;
		r[i] = bi;
		p[i] = zi;
		v[0] += bi * bi;
		v[1] += bi * zi;
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(v, part, &ctl->ticket[0], tot) && threadIdx.x == 0)
	{
		const double bb = tot[0];
		ctl->bb = bb;
		ctl->rz = tot[1];
		ctl->rr = bb;
		ctl->iter = 0;
		ctl->maxIter = maxIter;
		ctl->threshold = fmax(tol * tol * bb, DBL_MIN);
		ctl->converged = 1;
		ctl->done = (bb == 0.0 || bb < ctl->threshold) ? 1 : 0;
		if (!isfinite(bb))
		{
			ctl->done = 1;
			ctl->converged = 0;
		}
	}
}

// q = A p on the SELL-32 block matrix: one thread per block row (3 scalar rows), no reductions,
// every value and column load coalesced across the warp (a warp is one chunk).
__global__ void __launch_bounds__(256) k_cg_spmv_sell(MatSell3 A, const double* __restrict__ p,
													   double* __restrict__ q, CgCtl* ctl, double* part)
{
	if (ctl->done) return;
	double v[1] = {0.0};
	const int stride = gridDim.x * blockDim.x;
	const int nrowsPadded = (A.rows + 31) & ~31;
	for (int rs = blockIdx.x * blockDim.x + threadIdx.x; rs < nrowsPadded; rs += stride)
	{
		const int c = rs >> 5, lane = rs & 31;
		const int k0 = A.off[c], k1 = A.off[c + 1];
		double a0 = 0, a1 = 0, a2 = 0;
		for (int k = k0; k < k1; ++k)
		{
			const int J = A.col[k * 32 + lane];
			const double* vb = A.val + (size_t)k * 288 + lane;
			const double p0 = p[3 * J], p1 = p[3 * J + 1], p2 = p[3 * J + 2];
			a0 += vb[0] * p0 + vb[32] * p1 + vb[64] * p2;
			a1 += vb[96] * p0 + vb[128] * p1 + vb[160] * p2;
			a2 += vb[192] * p0 + vb[224] * p1 + vb[256] * p2;
		}
		if (rs < A.rows)
		{
			const int I = A.perm[rs];
			q[3 * I] = a0;
			q[3 * I + 1] = a1;
			q[3 * I + 2] = a2;
			v[0] += p[3 * I] * a0 + p[3 * I + 1] * a1 + p[3 * I + 2] * a2;
		}
	}
	double tot[1];
	if (grid_reduce<OpSum, 1>(v, part, &ctl->ticket[1], tot) && threadIdx.x == 0)
	{
		ctl->pq = tot[0];
		ctl->alpha = ctl->rz / tot[0];
	}
}

__global__ void __launch_bounds__(256) k_cg_spmv_csr(MatCsr A, const double* __restrict__ p, double* __restrict__ q,
													  CgCtl* ctl, double* part)
{
	if (ctl->done) return;
	const int lane = threadIdx.x & 31;
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int nwarps = (gridDim.x * blockDim.x) >> 5;
	double v[1] = {0.0};
	for (int row = warp; row < A.rows; row += nwarps)
	{
		double a = 0;
		for (int k = A.rowptr[row] + lane; k < A.rowptr[row + 1]; k += 32) a += A.val[k] * p[A.col[k]];
		a = warp_reduce<OpSum>(a);
		if (lane == 0)
		{
			q[row] = a;
			v[0] += p[row] * a;
		}
	}
	double tot[1];
	if (grid_reduce<OpSum, 1>(v, part, &ctl->ticket[1], tot) && threadIdx.x == 0)
	{
		ctl->pq = tot[0];
		ctl->alpha = ctl->rz / tot[0];
	}
}

__global__ void k_cg_update(int n, const double* __restrict__ invdiag, const double* __restrict__ p,
							const double* __restrict__ q, double* __restrict__ x, double* __restrict__ r, CgCtl* ctl,
							double* part)
{
	if (ctl->done) return;
	const double alpha = ctl->alpha;
	double v[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		x[i] += alpha * p[i];
		const double ri = r[i] - alpha * q[i];
		r[i] = ri;
		v[0] += ri * ri;
		v[1] += ri * (invdiag[i] * ri);
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(v, part, &ctl->ticket[2], tot) && threadIdx.x == 0)
	{
		const double rr = tot[0];
		ctl->rr = rr;
		if (rr < ctl->threshold)
		{
			ctl->done = 1;
			ctl->converged = 1;
		}
		else if (!isfinite(rr))
		{
			ctl->done = 1;  // a NaN residual never converges; stop instead of running to maxIter
			ctl->converged = 0;
		}
		else
		{
			const double rzOld = ctl->rz;
			ctl->rz = tot[1];
			ctl->beta = tot[1] / rzOld;
			ctl->iter += 1;
			if (ctl->iter >= ctl->maxIter)
			{
				ctl->done = 1;
				ctl->converged = 0;
			}
		}
	}
}

__global__ void k_cg_pupdate(int n, const double* __restrict__ invdiag, const double* __restrict__ r,
							 double* __restrict__ p, const CgCtl* ctl)
{
	if (ctl->done) return;
	const double beta = ctl->beta;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		p[i] = invdiag[i] * r[i] + beta * p[i];
}

// v_n += dv; x_n = x_t + dt v_n (OdeSolverEulerImplicit.cpp:98-99); optional Newton variation.
__global__ void k_state_update(int n, const double* __restrict__ dv, double* __restrict__ dvPrev,
							   const double* __restrict__ xt, double* __restrict__ xn, double* __restrict__ vn,
							   double dt, int trackNewton, CgCtl* ctl, double* part)
{
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double d = dv[i];
		const double vi = vn[i] + d;
		vn[i] = vi;
		xn[i] = xt[i] + dt * vi;
		if (trackNewton)
		{
			v[0] = fmax(v[0], fabs(d - dvPrev[i]));
			dvPrev[i] = d;
		}
	}
	if (!trackNewton) return;
	double tot[1];
	if (grid_reduce<OpMax, 1>(v, part, &ctl->ticket[3], tot) && threadIdx.x == 0) ctl->newtonVar = tot[0];
}

// OdeState::isValid: the sums of positions and of velocities are finite (OdeState.cpp:268-278).
__global__ void k_validity(int n, const double* __restrict__ x, const double* __restrict__ v, CgCtl* ctl, double* part)
{
	double s[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		s[0] += x[i];
		s[1] += v[i];
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(s, part, &ctl->ticket[3], tot) && threadIdx.x == 0)
	{
		ctl->sumX = tot[0];
		ctl->sumV = tot[1];
		ctl->nonfinite = !(isfinite(tot[0]) && isfinite(tot[1]));
	}
}

__global__ void k_scatter_values(int count, const int* __restrict__ idx, const double* __restrict__ vals,
								 double* __restrict__ dst)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < count) dst[idx[i]] = vals[i];
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
void launch_element_fp64(const DevBody& b, const double* xn, const double* vn, const double* xt, const double* vt,
						 double dt, double alpha, double beta, double* kslots, double* rhsE, double* kfull,
						 double* fE, int* counters, cudaStream_t s)
{
	if (b.E == 0) return;
	if (kfull)
		k_element_fp64<true><<<blocks(b.E, 64), 64, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE, kfull, fE,
															 counters);
	else
		k_element_fp64<false><<<blocks(b.E, 64), 64, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE, nullptr,
															  nullptr, counters);
}

void launch_assemble_bsr(const DevBody& b, const double* kslots, double c1, double c2, double* A, double* invdiag,
						 cudaStream_t s)
{
	if (b.nl == 0) return;
	k_assemble_bsr<<<blocks(b.nl, 128), 128, 0, s>>>(b, kslots, c1, c2, A, invdiag);
}

void launch_rhs_gather(const DevBody& b, const double* rhsE, const double* gravity, int gravityOn, double* rhs,
					   int applyBc, cudaStream_t s)
{
	if (b.N == 0) return;
	k_rhs_gather<<<blocks(b.N, 128), 128, 0, s>>>(b, rhsE, gravity[0], gravity[1], gravity[2], gravityOn, rhs, applyBc);
}

void launch_assemble_full_csc(int nnz, const int* sptr, const int* sidx, const int* srow, const int* scol,
							  const double* kfull, const double* smass, const uint8_t* bc, double c1, double c2,
							  double* S, cudaStream_t s)
{
	if (nnz == 0) return;
	k_assemble_full_csc<<<blocks(nnz, 256), 256, 0, s>>>(nnz, sptr, sidx, srow, scol, kfull, smass, bc, c1, c2, S);
}

void launch_cg_init(int n, const double* b, const double* invdiag, double* x, double* r, double* p, CgCtl* ctl,
					double* part, double tol, int maxIter, const Launch& L)
{
	k_cg_init<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, b, invdiag, x, r, p, ctl, part, tol, maxIter);
}

void launch_cg_spmv_sell(const MatSell3& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_spmv_sell<<<L.vecGrid, 256, 0, L.stream>>>(A, p, q, ctl, part);
}

void launch_cg_spmv_csr(const MatCsr& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_spmv_csr<<<L.vecGrid, 256, 0, L.stream>>>(A, p, q, ctl, part);
}

void launch_cg_update(int n, const double* invdiag, const double* p, const double* q, double* x, double* r,
					  CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_update<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invdiag, p, q, x, r, ctl, part);
}

void launch_cg_pupdate(int n, const double* invdiag, const double* r, double* p, CgCtl* ctl, const Launch& L)
{
	k_cg_pupdate<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invdiag, r, p, ctl);
}

void launch_state_update(int n, const double* dv, double* dvPrev, const double* xt, double* xn, double* vn,
						 double dt, int trackNewton, CgCtl* ctl, double* part, const Launch& L)
{
	k_state_update<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, dv, dvPrev, xt, xn, vn, dt, trackNewton, ctl, part);
}

void launch_validity(int n, const double* x, const double* v, CgCtl* ctl, double* part, const Launch& L)
{
	k_validity<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, x, v, ctl, part);
}

void launch_scatter_values(int count, const int* idx, const double* vals, double* dst, cudaStream_t s)
{
	if (count <= 0) return;
	k_scatter_values<<<blocks(count, 256), 256, 0, s>>>(count, idx, vals, dst);
}

}  // namespace gbfem
