// Test support only: the device element math of gbfem_element.cuh (and the element adjoint of
// gbfem_adjoint.cuh) compiled for the host, so the CPU test suite can compare it (FP64 and FP32)
// with the oracle element by element, and the adjoint with finite differences.
#include <type_traits>
#include <cmath>
#include <cstring>

#include "gbfem_adjoint.cuh"
#include "gbfem_element.cuh"

namespace {
double det33(const double m[3][3])
{
	return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
		   m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}
bool inverse44(const double a[4][4], double inv[4][4])
{
	double cof[4][4];
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j)
		{
			double m[3][3];
			int r = 0;
			for (int ii = 0; ii < 4; ++ii)
			{
				if (ii == i) continue;
				int c = 0;
				for (int jj = 0; jj < 4; ++jj)
					if (jj != j) m[r][c++] = a[ii][jj];
				++r;
			}
			cof[i][j] = (((i + j) & 1) ? -1.0 : 1.0) * det33(m);
		}
	double d = 0;
	for (int j = 0; j < 4; ++j) d += a[0][j] * cof[0][j];
	if (!(std::fabs(d) > 1e-12)) return false;
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j) inv[i][j] = cof[j][i] / d;
	return true;
}
double det3v(const double* a, const double* b, const double* c)
{
	return a[0] * b[1] * c[2] + a[2] * b[0] * c[1] + a[1] * b[2] * c[0] - a[2] * b[1] * c[0] - a[1] * b[0] * c[2] -
		   a[0] * b[2] * c[1];
}

template <typename T>
int run(const double* x0, const double* x, const double* v, const double* xt, const double* vt, const int* nd,
		double E, double nu, double rho, double dt, double alpha, double beta, double* K, double* rhs, double* f,
		double* R9)
{
	double V[4][4], Vi[4][4];
	for (int a = 0; a < 4; ++a)
	{
		for (int k = 0; k < 3; ++k) V[k][a] = x0[3 * a + k];
		V[3][a] = 1.0;
	}
	if (!inverse44(V, Vi)) return -1;
	const double vol = (det3v(x0 + 3, x0 + 6, x0 + 9) - det3v(x0, x0 + 6, x0 + 9) + det3v(x0, x0 + 3, x0 + 9) -
						det3v(x0, x0 + 3, x0 + 6)) / 6.0;
	const double lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
	const double mu = E / (2.0 * (1 + nu));
	gbfem::elem::ElemIn in;
	for (int a = 0; a < 4; ++a)
	{
		in.nd[a] = nd[a];
		for (int k = 0; k < 3; ++k)
		{
			in.p[a][k] = x[3 * a + k] - x[k];
			in.q[a][k] = x0[3 * a + k] - x0[k];
			const double va = v[3 * a + k];
			in.uK[a][k] = -beta * va + ((x[3 * a + k] - xt[3 * a + k]) - dt * va);
			in.uM[a][k] = -alpha * va - (va - vt[3 * a + k]) / dt;
			in.vv[a][k] = va;
		}
	}
	in.alphaDbg = alpha;
	in.betaDbg = beta;
	T g[4][3];
	for (int a = 0; a < 4; ++a)
		for (int k = 0; k < 3; ++k) g[a][k] = T(Vi[a][k]);
	T ks[90], rh[12];
	double fd[12];
	int fl = gbfem::elem::compute<T, true>(in, g, T(lambda * vol), T(mu * vol), T(vol * rho / 20.0), ks, 1, rh, 1, K,
										   fd);
	for (int i = 0; i < 12; ++i)
	{
		rhs[i] = double(rh[i]);
		f[i] = fd[i];
	}
	// R from the Newton polar (or its fallback) on the same F
	T F[9], Rt[9];
	gbfem::elem::deformation<T, false>(in, g, F);
	gbfem::elem::rotation<T, false>(in, g, F, Rt);
	for (int k = 0; k < 9; ++k) R9[k] = double(Rt[k]);
	return fl;
}
}  // namespace

extern "C" int gbfem_host_element(int fp32, const double* x0, const double* x, const double* v, const double* xt,
								  const double* vt, const int* nd, double E, double nu, double rho, double dt,
								  double alpha, double beta, double* K144, double* rhs12, double* f12, double* R9)
{
	return fp32 ? run<float>(x0, x, v, xt, vt, nd, E, nu, rho, dt, alpha, beta, K144, rhs12, f12, R9)
				: run<double>(x0, x, v, xt, vt, nd, E, nu, rho, dt, alpha, beta, K144, rhs12, f12, R9);
}

// psi_e and its derivatives for one element (x, v absolute positions / velocities of the 4 nodes,
// mu and dv the adjoint and velocity increment at its 12 dofs). Returns -1 for a degenerate rest tet.
extern "C" int gbfem_host_adjoint_element(const double* x0, const double* x, const double* v, const int* nd, double E,
										  double nu, double rho, double dt, double alpha, double beta, const double* mu,
										  const double* dv, double* psi, double* gx, double* gv, double* pLam,
										  double* pMu)
{
	double V[4][4], Vi[4][4];
	for (int a = 0; a < 4; ++a)
	{
		for (int k = 0; k < 3; ++k) V[k][a] = x0[3 * a + k];
		V[3][a] = 1.0;
	}
	if (!inverse44(V, Vi)) return -1;
	const double vol = (det3v(x0 + 3, x0 + 6, x0 + 9) - det3v(x0, x0 + 6, x0 + 9) + det3v(x0, x0 + 3, x0 + 9) -
						det3v(x0, x0 + 3, x0 + 6)) / 6.0;
	const double lambda = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
	const double mu_ = E / (2.0 * (1 + nu));
	int ndv[4];
	double X[4][3], R0[4][3], Vel[4][3], MU[12], DV[12], g[4][3];
	for (int a = 0; a < 4; ++a)
	{
		ndv[a] = nd[a];
		for (int k = 0; k < 3; ++k)
		{
			X[a][k] = x[3 * a + k];
			R0[a][k] = x0[3 * a + k];
			Vel[a][k] = v[3 * a + k];
			g[a][k] = Vi[a][k];
		}
	}
	for (int j = 0; j < 12; ++j)
	{
		MU[j] = mu[j];
		DV[j] = dv[j];
	}
	const double lamV = lambda * vol, muV = mu_ * vol, cm = vol * rho / 20.0;
	gbfem::elem::ElemIn in;
	gbfem::adj::fill_input(in, ndv, X, R0, Vel, dt, alpha, beta, -1, -1);
	double ks[90], rh[12];
	gbfem::elem::compute<double, false>(in, g, lamV, muV, cm, ks, 1, rh, 1, nullptr, nullptr);
	// psi_e two ways: contracted as the element code delivers its blocks (what the derivative passes
	// differentiate) and from the stored blocks; they agree to rounding.
	*psi = gbfem::adj::element_psi_value(ndv, X, R0, Vel, MU, DV, g, lamV, muV, cm, dt, alpha, beta);
	const double psiArrays = gbfem::adj::element_psi(ndv, ks, rh, MU, DV, dt + beta);
	double scale = 0.0, mmax = 0.0, dmax = 0.0;
	for (int j = 0; j < 12; ++j)
	{
		scale += fabs(MU[j] * rh[j]);
		mmax = fmax(mmax, fabs(MU[j]));
		dmax = fmax(dmax, fabs(DV[j]));
	}
	for (int k = 0; k < 90; ++k) scale += 2.0 * (dt + beta) * fabs(ks[k]) * mmax * dmax;
	if (!(fabs(*psi - psiArrays) <= 1e-13 * scale)) return -2;
	gbfem::adj::element_adjoint<double>(ndv, X, R0, Vel, MU, DV, g, lamV, muV, cm, dt, alpha, beta, gx, gv, pLam, pMu);
	return 0;
}

// d(lambda V)/d nu and d(mu V)/d nu as the adjoint kernel forms them from the stored moduli.
extern "C" void gbfem_host_poisson_partials(double lamV, double muV, double* dLam, double* dMu)
{
	gbfem::adj::poisson_partials(lamV, muV, dLam, dMu);
}
