// gbfem_adjoint.cuh -- per-element derivatives of one implicit-Euler step (host and device).
//
// psi_e(x_e, v_e, lambda V, mu V) = mu_e . rhs_e - c2 <lower-triangle blocks of K_e, (mu, dv)> is the
// element's share of psi = mu . rhs - mu . S dv, the scalar whose gradients give the step's adjoint
// (see gbfem_adjoint.cu). adjoint_element() returns d psi_e / d x_e (12, forward-mode dual
// numbers through the element code, nine passes), d psi_e / d v_e (12) and d psi_e / d(lambda V), d(mu V).
#pragma once

#include "gbfem_element.cuh"

namespace gbfem {
namespace adj {

// psi_e = mu_e . rhs_e - c2 <K_e's lower-triangle blocks, (mu, dv)>; the stored blocks are the
// element's diagonal node blocks (read lower-triangular, like the assembled matrix) and, per node
// pair, the block whose row node has the larger id.
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

template <typename P>
__host__ __device__ void fill_input(elem::ElemInT<P>& in, const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
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
			in.q[a][k] = P(R0[a][k] - R0[0][k]);
			const double va = V[a][k];
			in.uK[a][k] = P(-beta * va + (0.0 - dt * va));  // x_n = x_t at the first Newton iteration
			in.uM[a][k] = P(-alpha * va);                    // v_n = v_t
			in.vv[a][k] = P(va);
		}
	}
	in.alphaDbg = alpha;
	in.betaDbg = beta;
}

// Work items of one element, each an independent pass through the element code: items 0..8 are the
// dual passes seeded on x_(1 + item/3, item%3) (psi_e depends on the positions only through
// p_a = x_a - x_0, so d/dx_0 = -sum_a d/dx_a needs no pass of its own), item 9 the velocity
// gradient, item 10 the two unit-modulus evaluations.
constexpr int kAdjItems = 11;

// One item of one element: X, R0, V positions / rest positions / velocities of its nodes, MU and DV
// the adjoint and the step's velocity increment at its dofs (zero on BC dofs). Writes gx[3 + item]
// (items 0..8), gv[0..11] (item 9) or *pLam, *pMu (item 10).
// S is the arithmetic of the passes: double (FP64 form) or float (mixed form, FP32 element math
// with the corotated strain formed as in its forward step).
template <typename S = double>
__host__ __device__ inline void adjoint_item(int item, const int (&nd)[4], const double (&X)[4][3],
											 const double (&R0)[4][3], const double (&V)[4][3], const double (&MU)[12],
											 const double (&DV)[12], const double (&g)[4][3], double lamV, double muV,
											 double cm, double dt, double alpha, double beta, double* gx, double* gv,
											 double* pLam, double* pMu, bool lumped = false)
{
	using D = ad::DualT<S>;
	const double c2 = dt + beta;
	if (item < 9)
	{
		D gD[4][3];
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) gD[a][k] = D(g[a][k]);
		const int s = 3 + item;
		elem::ElemInT<D> in;
		fill_input(in, nd, X, R0, V, dt, alpha, beta, s / 3, s % 3, lumped);
		D ks[kSlots * 9], rhs[12];
		elem::compute<D, false, elem::ElemInT<D>>(in, gD, D(lamV), D(muV), D(cm), ks, 1, rhs, 1, nullptr, nullptr);
		gx[s] = double(element_psi(nd, ks, rhs, MU, DV, c2).d);
	}
	else if (item == 9)
	{
		// d psi_e / d v_e = -c2 K_e^T mu_e - alpha M0 mu_e (K_e: the full element tangent; M0 lumped to
		// 5 cm on the diagonal with mass lumping).
		elem::ElemIn in;
		fill_input(in, nd, X, R0, V, dt, alpha, beta, -1, -1, lumped);
		S gS[4][3], ks[kSlots * 9], rhs[12];
		double kfull[144], fdbg[12];
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) gS[a][k] = S(g[a][k]);
		elem::compute<S, true>(in, gS, S(lamV), S(muV), S(cm), ks, 1, rhs, 1, kfull, fdbg);
		double sm[3] = {0, 0, 0};
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) sm[k] += MU[3 * a + k];
		for (int c = 0; c < 12; ++c)
		{
			double t = 0.0;
			for (int r = 0; r < 12; ++r) t += kfull[r * 12 + c] * MU[r];
			gv[c] = -c2 * t - alpha * cm * (lumped ? 5.0 * MU[c] : MU[c] + sm[c % 3]);
		}
	}
	else
	{
		// psi_e's elastic part is linear in (lambda V, mu V): evaluate it with unit moduli.
		elem::ElemIn in;
		fill_input(in, nd, X, R0, V, dt, alpha, beta, -1, -1);
		S gS[4][3], ks[kSlots * 9], rhs[12];
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) gS[a][k] = S(g[a][k]);
		elem::compute<S, false>(in, gS, S(1), S(0), S(0), ks, 1, rhs, 1, nullptr, nullptr);
		*pLam = double(element_psi(nd, ks, rhs, MU, DV, c2));
		elem::compute<S, false>(in, gS, S(0), S(1), S(0), ks, 1, rhs, 1, nullptr, nullptr);
		*pMu = double(element_psi(nd, ks, rhs, MU, DV, c2));
	}
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

// All items of one element in one call (gx[0..2] completed from translation invariance).
__host__ __device__ inline void adjoint_element(const int (&nd)[4], const double (&X)[4][3], const double (&R0)[4][3],
												const double (&V)[4][3], const double (&MU)[12], const double (&DV)[12],
												const double (&g)[4][3], double lamV, double muV, double cm, double dt,
												double alpha, double beta, double* gx, double* gv, double* pLam,
												double* pMu, bool lumped = false)
{
	for (int item = 0; item < kAdjItems; ++item)
		adjoint_item(item, nd, X, R0, V, MU, DV, g, lamV, muV, cm, dt, alpha, beta, gx, gv, pLam, pMu, lumped);
	for (int k = 0; k < 3; ++k) gx[k] = -(gx[3 + k] + gx[6 + k] + gx[9 + k]);
}

}  // namespace adj
}  // namespace gbfem
