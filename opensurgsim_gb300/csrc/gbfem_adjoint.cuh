// gbfem_adjoint.cuh -- per-element derivatives of one implicit-Euler step (host and device).
//
// psi_e(x_e, v_e, lambda V, mu V) = mu_e . rhs_e - c2 <lower-triangle blocks of K_e, (mu, dv)> is the
// element's share of psi = mu . rhs - mu . S dv, the scalar whose gradients give the step's adjoint
// (see gbfem_adjoint.cu). element_adjoint() returns d psi_e / d x_e (12, forward-mode dual
// numbers through the element code, nine passes), d psi_e / d v_e (12) and d psi_e / d(lambda V), d(mu V).
#pragma once

#include "gbfem_element.cuh"

namespace gbfem {
namespace adj {

// psi_e = mu_e . rhs_e - c2 <K_e's lower-triangle blocks, (mu, dv)>; the stored blocks are the
// element's diagonal node blocks (read lower-triangular, like the assembled matrix) and, per node
// pair, the block whose row node has the larger id. This form reads stored arrays (host checks);
// the adjoint kernel contracts the blocks as the element code produces them (PsiOut).
template <typename T>
__host__ __device__ T element_psi(const int (&nd)[4], const T* ks, const T* rhs, const double (&mu)[12], const double (&dv)[12],
						 double c2)
{
	T s = T(0);
#pragma unroll
	for (int j = 0; j < 12; ++j) s += T(mu[j]) * rhs[j];
	T sk = T(0);
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j <= i; ++j)
			{
				const double c = mu[3 * a + i] * dv[3 * a + j] + (i != j ? mu[3 * a + j] * dv[3 * a + i] : 0.0);
				sk += ks[a * 9 + 3 * i + j] * T(c);
			}
#pragma unroll
	for (int lo = 0; lo < 4; ++lo)
#pragma unroll
		for (int hi = lo + 1; hi < 4; ++hi)
		{
			const int slot = elem::pair_slot(lo, hi);
			const int r = (nd[lo] > nd[hi]) ? lo : hi, cc = (r == lo) ? hi : lo;
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
				{
					const double c = mu[3 * r + i] * dv[3 * cc + j] + mu[3 * cc + j] * dv[3 * r + i];
					sk += ks[slot * 9 + 3 * i + j] * T(c);
				}
		}
	return s - T(c2) * sk;
}

// The two sums of psi_e = s - c2 sk, accumulated as compute_to() delivers the element's right-hand
// side (s = mu_e . rhs_e) and stored blocks (sk, the coefficients of element_psi), so that no block
// is held: an output policy of compute_to().
template <typename T>
struct PsiOut
{
	using G = typename elem::ScalarOf<T>::type;
	const G (&mu)[12];  // in the passes' arithmetic (FP32 for the mixed form's passes)
	const G (&dv)[12];
	T s = T(0), sk = T(0);
	static constexpr bool kAll = false;
	__host__ __device__ __forceinline__ PsiOut(const G (&MU)[12], const G (&DV)[12]) : mu(MU), dv(DV) {}
	__host__ __device__ __forceinline__ bool blocks() const { return true; }
	__host__ __device__ __forceinline__ void rhs_entry(int j, const T& v) { s = s + v * mu[j]; }
	__host__ __device__ __forceinline__ void block(int a, int b, int, const T (&blk)[9])
	{
		if (a == b)
		{
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j <= i; ++j)
				{
					const G c = mu[3 * a + i] * dv[3 * a + j] + (i != j ? mu[3 * a + j] * dv[3 * a + i] : G(0));
					sk = sk + blk[3 * i + j] * c;
				}
		}
		else
		{
#pragma unroll
			for (int i = 0; i < 3; ++i)
#pragma unroll
				for (int j = 0; j < 3; ++j)
				{
					const G c = mu[3 * a + i] * dv[3 * b + j] + mu[3 * b + j] * dv[3 * a + i];
					sk = sk + blk[3 * i + j] * c;
				}
		}
	}
	__host__ __device__ __forceinline__ void full_block(int, int, const T (&)[9]) {}
	__host__ __device__ __forceinline__ T psi(double c2) const { return s - G(c2) * sk; }
};

// (K_e^T mu_e)_c = sum_r K_e(r, c) mu_r over the full element tangent, accumulated in r order in the
// passes' arithmetic as compute_to() delivers its 16 blocks: an output policy of compute_to().
template <typename T>
struct KtMuOut
{
	const T (&mu)[12];
	T kt[12] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
	static constexpr bool kAll = true;
	__host__ __device__ __forceinline__ KtMuOut(const T (&MU)[12]) : mu(MU) {}
	__host__ __device__ __forceinline__ bool blocks() const { return false; }
	__host__ __device__ __forceinline__ void rhs_entry(int, const T&) {}
	__host__ __device__ __forceinline__ void block(int, int, int, const T (&)[9]) {}
	__host__ __device__ __forceinline__ void full_block(int a, int b, const T (&blk)[9])
	{
#pragma unroll
		for (int q = 0; q < 3; ++q)
#pragma unroll
			for (int i = 0; i < 3; ++i) kt[3 * b + q] += blk[3 * i + q] * mu[3 * a + i];
	}
};

// psi_e's sums and K_e^T mu_e from the same pass: an output policy of compute_to().
template <typename T>
struct PsiKtOut
{
	PsiOut<T> psi;
	KtMuOut<T> kt;
	static constexpr bool kAll = true;
	__host__ __device__ __forceinline__ PsiKtOut(const T (&MU)[12], const T (&DV)[12]) : psi(MU, DV), kt(MU) {}
	__host__ __device__ __forceinline__ bool blocks() const { return true; }
	__host__ __device__ __forceinline__ void rhs_entry(int j, const T& v) { psi.rhs_entry(j, v); }
	__host__ __device__ __forceinline__ void block(int a, int b, int slot, const T (&blk)[9]) { psi.block(a, b, slot, blk); }
	__host__ __device__ __forceinline__ void full_block(int a, int b, const T (&blk)[9]) { kt.full_block(a, b, blk); }
};

template <typename P, typename C>
__host__ __device__ void fill_input(elem::ElemInT<P, C>& in, const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
						   const double (&V)[4][3], double dt, double alpha, double beta, int seedNode, int seedAxis,
						   bool lumped = false)
{
	in.lumped = lumped ? 1 : 0;
#pragma unroll
	for (int a = 0; a < 4; ++a)
	{
		in.nd[a] = nd[a];
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			// p_a = x_a - x_0; its derivative along x_(seedNode, seedAxis).
			const double dp = (k == seedAxis) ? (double(a == seedNode) - double(seedNode == 0)) : 0.0;
			in.p[a][k] = P(X[a][k] - X[0][k]);
			if constexpr (!std::is_same<P, double>::value) in.p[a][k].d = dp;
			in.q[a][k] = C(R0[a][k] - R0[0][k]);
			const double va = V[a][k];
			in.uK[a][k] = C(-beta * va + (0.0 - dt * va));  // x_n = x_t at the first Newton iteration
			in.uM[a][k] = C(-alpha * va);                    // v_n = v_t
			in.vv[a][k] = C(va);
		}
	}
	in.alphaDbg = alpha;
	in.betaDbg = beta;
}

// The element's rotation in the passes' arithmetic S (row-major) and its polar flags, as the
// element code forms them: computed once and shared by every pass over the element.
template <typename S = double>
__host__ __device__ inline int element_rotation(const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
												const double (&g)[4][3], S (&R)[9])
{
	elem::ElemIn in;
	const double zero[4][3] = {};
	fill_input(in, nd, X, R0, zero, 0.0, 0.0, 0.0, -1, -1);
	S gS[4][3], F[9];
	for (int a = 0; a < 4; ++a)
		for (int k = 0; k < 3; ++k) gS[a][k] = S(g[a][k]);
	elem::deformation<S, false>(in, gS, F);
	return elem::rotation<S, false>(in, gS, F, R);
}

// All derivatives of psi_e for one element. X, R0, V: positions / rest positions / velocities of its
// nodes; MU, DV: the adjoint and the step's velocity increment at its dofs (zero on BC dofs).
//   gx[0..11] = d psi_e / d x_e: nine dual passes seeded on x_(b, k), b = 1..3 (psi_e depends on the
//     positions only through p_a = x_a - x_0, so d/dx_0 = -sum_b d/dx_b needs no pass of its own);
//   gv[0..11] = d psi_e / d v_e = -c2 K_e^T mu_e - alpha M0 mu_e (M0 lumped to 5 cm on the diagonal
//     with mass lumping);
//   *pLam, *pMu (when pLam is not null) = psi_e's elastic part at unit (lambda V, mu V), in which it is
//     linear; the same two passes give K_e^T mu_e.
// S is the arithmetic of the passes: double (FP64 form) or float (mixed form, FP32 element math
// with the corotated strain formed as in its forward step). The rotation, the passes' inputs and the
// psi coefficients are formed once; a dual pass only moves its seed.
template <typename S = double>
__host__ __device__ inline void element_adjoint(const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
												const double (&V)[4][3], const double (&MU)[12], const double (&DV)[12],
												const double (&g)[4][3], double lamV, double muV, double cm, double dt,
												double alpha, double beta, double* gx, double* gv, double* pLam,
												double* pMu, bool lumped = false)
{
	using D = ad::DualT<S>;
	const double c2 = dt + beta;
	S Rw[9];
	const int rflags = element_rotation<S>(nd, X, R0, g, Rw);
	S gS[4][3], muS[12], dvS[12];
	for (int a = 0; a < 4; ++a)
		for (int k = 0; k < 3; ++k) gS[a][k] = S(g[a][k]);
	for (int j = 0; j < 12; ++j)
	{
		muS[j] = S(MU[j]);
		dvS[j] = S(DV[j]);
	}
	{
		// Positions: only they carry the seeded derivative (the rotation's from polar_tangent); psi_e's
		// sums are contracted as the blocks come out of the element code. One body for the nine
		// passes (a loop, not unrolled).
		elem::ElemInT<D, S> in;
		fill_input(in, nd, X, R0, V, dt, alpha, beta, -1, -1, lumped);
		double sx[3] = {0.0, 0.0, 0.0};
#pragma unroll 1
		for (int item = 0; item < 9; ++item)
		{
			const int node = 1 + item / 3, axis = item % 3;
#pragma unroll
			for (int a = 0; a < 4; ++a)
#pragma unroll
				for (int k = 0; k < 3; ++k) in.p[a][k].d = (a == node && k == axis) ? S(1) : S(0);
			PsiOut<D> out(muS, dvS);
			elem::compute_to<D, false, elem::ElemInT<D, S>, false>(in, gS, S(lamV), S(muV), S(cm), out, nullptr,
																   nullptr, Rw, rflags);
			const double d = double(out.psi(c2).d);
			gx[3 + item] = d;
			sx[axis] += d;
		}
		for (int k = 0; k < 3; ++k) gx[k] = -sx[k];
	}
	{
		// psi_e's elastic part and K_e are linear in (lambda V, mu V) (K0, the rotated stiffness and the
		// rotation terms all are; R and the singular-G decision do not depend on the moduli): two passes
		// at unit moduli (mass terms off, cm = 0) give d psi_e / d(lambda V), d(mu V) and
		// K_e^T mu_e = lambda V K_lam^T mu_e + mu V K_mu^T mu_e.
		elem::ElemIn in;
		fill_input(in, nd, X, R0, V, dt, alpha, beta, -1, -1, lumped);
		double pu[2], kt[12];
		for (int c = 0; c < 12; ++c) kt[c] = 0.0;
		// FP32 passes: one loop body (the kernel's size costs more than the unit moduli folded in);
		// FP64 passes, bound by the FP64 rate: unrolled, with the unit moduli folded.
		constexpr int kUnroll = std::is_same<S, float>::value ? 1 : 2;
#pragma unroll kUnroll
		for (int u = 0; u < 2; ++u)
		{
			PsiKtOut<S> out(muS, dvS);
			elem::compute_to<S, false, elem::ElemIn, false, PsiKtOut<S>, true>(in, gS, S(u == 0 ? 1 : 0), S(u == 0 ? 0 : 1),
																				S(0), out, nullptr, nullptr, Rw, rflags);
			pu[u] = double(out.psi.psi(c2));
			const double m = (u == 0) ? lamV : muV;
			for (int c = 0; c < 12; ++c) kt[c] += m * double(out.kt.kt[c]);
		}
		double sm[3] = {0, 0, 0};
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) sm[k] += MU[3 * a + k];
		for (int c = 0; c < 12; ++c)
			gv[c] = -c2 * kt[c] - alpha * cm * (lumped ? 5.0 * MU[c] : MU[c] + sm[c % 3]);
		if (pLam)
		{
			*pLam = pu[0];
			*pMu = pu[1];
		}
	}
}

// psi_e itself in FP64 (host checks of its derivatives), through the same contraction as the
// derivative passes.
__host__ __device__ inline double element_psi_value(const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
													const double (&V)[4][3], const double (&MU)[12], const double (&DV)[12],
													const double (&g)[4][3], double lamV, double muV, double cm, double dt,
													double alpha, double beta, bool lumped = false)
{
	elem::ElemIn in;
	fill_input(in, nd, X, R0, V, dt, alpha, beta, -1, -1, lumped);
	PsiOut<double> out(MU, DV);
	elem::compute_to<double, false, elem::ElemIn, false>(in, g, lamV, muV, cm, out, nullptr, nullptr);
	return out.psi(dt + beta);
}

// Chain rule from the element's moduli to its Poisson ratio: with lambda V = V E nu / ((1 + nu)
// (1 - 2 nu)) and mu V = V E / (2 (1 + nu)) (Fem3DElementTetrahedron.cpp:204-205) at fixed E,
// d(lambda V)/d nu = V E (1 + 2 nu^2) / ((1 + nu)^2 (1 - 2 nu)^2) and d(mu V)/d nu = -V E / (2 (1 + nu)^2);
// nu = lambda / (2 (lambda + mu)) and V E = 2 mu V (1 + nu) are recovered from the stored moduli.
__host__ __device__ inline void poisson_partials(double lamV, double muV, double* dLam, double* dMu)
{
	const double nu = lamV / (2.0 * (lamV + muV));
	const double EV = 2.0 * muV * (1.0 + nu);
	*dLam = EV * (1.0 + 2.0 * nu * nu) / ((1.0 + nu) * (1.0 + nu) * (1.0 - 2.0 * nu) * (1.0 - 2.0 * nu));
	*dMu = -EV / (2.0 * (1.0 + nu) * (1.0 + nu));
}

}  // namespace adj
}  // namespace gbfem
