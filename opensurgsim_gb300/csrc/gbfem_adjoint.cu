// gbfem_adjoint.cu -- reverse-mode derivative of one implicit-Euler step (the differentiation form).
//
// Forward step at state (x, v) (one Newton iteration, OdeSolverEulerImplicit.cpp:55-161):
//   S(x) dv = rhs(x, v),  v' = v + dv,  x' = x + dt v'
// with rhs = sum_e [f_e(x) - c2 K_e(x) v - alpha M_e v] + gravity, S = c1 M + c2 K(x) read through
// its lower triangle (the CG's SelfAdjointView<Lower>), BC rows/columns fixed. Given the loss
// gradients (lx, lv) = (dL/dx', dL/dv'), the step's adjoint is
//   S mu = dt lx + lv                    (the transposed solve; S is symmetric as the CG reads it)
//   dL/dx   = lx + grad_x psi,  dL/dv = dt lx + lv + grad_v psi,  dL/dtheta_e = d psi / d theta_e
// where psi(x, v, theta) = mu . rhs - mu . S dv (mu and dv held fixed; BC entries of both are zero,
// which removes the BC rows and columns the forward replaces by constants). psi is a sum of
// element terms psi_e, so the per-element kernels below produce d psi_e / d(x_e, v_e, E_e, nu_e):
//   - x: forward-mode dual numbers through the same element code (9 seeded passes; FP64 for the
//     FP64 form, FP32 for the mixed form, whose forward element math is FP32 too), which
//     differentiates the rotation, the corotated tangent (its dR/dx terms) and the force exactly;
//   - v: psi is linear in v, d psi_e / d v_e = -c2 K_e^T mu_e - alpha M0 mu_e (M0 lumped with mass
//     lumping);
//   - E, nu: psi_e is linear in (lambda V, mu V), so two evaluations with unit moduli give both.

#include "gbfem_adjoint.cuh"
#include "gbfem_internal.h"

namespace gbfem {
namespace {

constexpr int kAdjThreads = 64;

// One thread per element, its passes in turn (splitting them over threads was measured slower:
// every pass needs the same large per-thread state). gx[e*12 + 0..11], gv[e*12 + 0..11]; gLogE[e],
// gNu[e] accumulate.
template <typename S>
__global__ void __launch_bounds__(kAdjThreads) k_element_adjoint(DevBody b, const double* __restrict__ x,
																 const double* __restrict__ v,
																 const double* __restrict__ mu,
																 const double* __restrict__ dv, double dt, double alpha,
																 double beta, double* __restrict__ gx,
																 double* __restrict__ gv, double* __restrict__ gLogE,
																 double* __restrict__ gNu)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= b.E) return;
	const int E = b.E;
	const int4 t4 = b.tets[e];
	const int nd[4] = {t4.x, t4.y, t4.z, t4.w};
	double X[4][3], R0[4][3], V[4][3], MU[12], DV[12];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			const int d = 3 * nd[a] + k;
			X[a][k] = x[d];
			R0[a][k] = b.xrest[d];
			V[a][k] = v[d];
			MU[3 * a + k] = b.bc[d] ? 0.0 : mu[d];
			DV[3 * a + k] = b.bc[d] ? 0.0 : dv[d];
		}
	double g[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k) g[a][k] = b.rest[(3 * a + k) * E + e];
	const double lamV = b.rest[13 * E + e], muV = b.rest[14 * E + e], cm = b.rest[15 * E + e];
	const bool moduli = gLogE || gNu;
	double pl = 0.0, pm = 0.0;
	adj::element_adjoint<S>(nd, X, R0, V, MU, DV, g, lamV, muV, cm, dt, alpha, beta, gx + (size_t)e * 12,
							gv + (size_t)e * 12, moduli ? &pl : nullptr, &pm, b.lumped != 0);
	if (!moduli) return;
	// lambda V and mu V are both proportional to E: d/d log E scales each by one.
	if (gLogE) gLogE[e] += lamV * pl + muV * pm;
	if (gNu)
	{
		double dl, dm;
		adj::poisson_partials(lamV, muV, &dl, &dm);
		gNu[e] += dl * pl + dm * pm;
	}
}

// dL/dx_t = lx + sum_e gx, dL/dv_t = dt lx + lv + sum_e gv, summed over each node's incidences in
// element order (deterministic); an element's node 0 takes minus the sum of its nodes 1..3.
__global__ void k_adjoint_gather(DevBody b, const double* __restrict__ gx, const double* __restrict__ gv,
								 const double* __restrict__ lx, const double* __restrict__ lv, double dt,
								 double* __restrict__ lxOut, double* __restrict__ lvOut)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= b.N) return;
	double sx[3] = {0, 0, 0}, sv[3] = {0, 0, 0};
	const int k1 = b.iptr[I + 1];
	for (int k = b.iptr[I]; k < k1; ++k)
	{
		const int c = b.iidx[k];
		const size_t o = (size_t)(c >> 2) * 12;
		const int a = c & 3;
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			sx[j] += (a == 0) ? -(gx[o + 3 + j] + gx[o + 6 + j] + gx[o + 9 + j]) : gx[o + 3 * a + j];
			sv[j] += gv[o + 3 * a + j];
		}
	}
#pragma unroll
	for (int j = 0; j < 3; ++j)
	{
		const int d = 3 * I + j;
		const double l = lx[d];
		lxOut[d] = l + sx[j];
		lvOut[d] = dt * l + lv[d] + sv[j];
	}
}

// Right-hand side of the transposed solve, g = dt lx + lv, zero on BC dofs.
__global__ void k_adjoint_rhs(int n, const uint8_t* __restrict__ bc, const double* __restrict__ lx,
							  const double* __restrict__ lv, double dt, double* __restrict__ g)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) g[i] = bc[i] ? 0.0 : dt * lx[i] + lv[i];
}

// Per-element moduli: lambda V and mu V from E and nu (the host passes its stored per-element nu when
// the caller gives none; deriving nu from the rounded lambda V, mu V would drift it call by call).
__global__ void k_set_materials(int E, const double* __restrict__ young, const double* __restrict__ poisson,
								double* __restrict__ rest, float* __restrict__ rest32)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= E) return;
	const double vol = rest[12 * (size_t)E + e];
	const double nu =
		poisson ? poisson[e] : rest[13 * (size_t)E + e] / (2.0 * (rest[13 * (size_t)E + e] + rest[14 * (size_t)E + e]));
	const double Ey = young[e];
	const double lambda = Ey * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
	const double mu = Ey / (2.0 * (1 + nu));
	rest[13 * (size_t)E + e] = lambda * vol;
	rest[14 * (size_t)E + e] = mu * vol;
	if (rest32)
	{
		rest32[13 * (size_t)E + e] = float(lambda * vol);
		rest32[14 * (size_t)E + e] = float(mu * vol);
	}
}

inline int blocks_of(long long n, int t) { return (int)((n + t - 1) / t); }

__global__ void k_vec_diff(int n, const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = a[i] - b[i];
}

}  // namespace

void launch_vec_diff(int n, const double* a, const double* b, double* out, cudaStream_t s)
{
	if (n == 0) return;
	k_vec_diff<<<blocks_of(n, 256), 256, 0, s>>>(n, a, b, out);
}

void launch_element_adjoint(const DevBody& b, const double* x, const double* v, const double* mu, const double* dv,
							double dt, double alpha, double beta, double* gx, double* gv, double* gLogE, double* gNu,
							cudaStream_t s, bool fp32)
{
	if (b.E == 0) return;
	if (fp32)
		k_element_adjoint<float><<<blocks_of(b.E, kAdjThreads), kAdjThreads, 0, s>>>(b, x, v, mu, dv, dt, alpha, beta,
																					 gx, gv, gLogE, gNu);
	else
		k_element_adjoint<double><<<blocks_of(b.E, kAdjThreads), kAdjThreads, 0, s>>>(b, x, v, mu, dv, dt, alpha, beta,
																					  gx, gv, gLogE, gNu);
}

void launch_adjoint_gather(const DevBody& b, const double* gx, const double* gv, const double* lx, const double* lv,
						   double dt, double* lxOut, double* lvOut, cudaStream_t s)
{
	if (b.N == 0) return;
	k_adjoint_gather<<<blocks_of(b.N, 128), 128, 0, s>>>(b, gx, gv, lx, lv, dt, lxOut, lvOut);
}

void launch_adjoint_rhs(int n, const uint8_t* bc, const double* lx, const double* lv, double dt, double* g,
						cudaStream_t s)
{
	if (n == 0) return;
	k_adjoint_rhs<<<blocks_of(n, 256), 256, 0, s>>>(n, bc, lx, lv, dt, g);
}

void launch_set_materials(int E, const double* young, const double* poisson, double* rest, float* rest32,
						  cudaStream_t s)
{
	if (E == 0) return;
	k_set_materials<<<blocks_of(E, 256), 256, 0, s>>>(E, young, poisson, rest, rest32);
}

}  // namespace gbfem
