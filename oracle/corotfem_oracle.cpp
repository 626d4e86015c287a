// corotfem_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU, FP64 restatement of OpenSurgSim's corotational-tetrahedron implicit-Euler step
// (Fem3DRepresentation + Fem3DElementCorotationalTetrahedron + OdeSolverEulerImplicit +
// LinearSparseSolveAndInverseCG). It is the parity checker for the CUDA library and the timed
// CPU baseline; nothing in the product links it. Every routine cites the reference file:line
// it restates (paths relative to the OpenSurgSim source tree).
//
// Eigen is not available, so the three Eigen features the path relies on are restated from
// their published definitions:
//   * Eigen::ConjugateGradient<SparseMatrix<double>, Lower, DiagonalPreconditioner>
//     (LinearSparseSolveAndInverse.h:122): zero initial guess, Jacobi preconditioner
//     (1/diag, 1 where the diagonal is 0), only the lower triangle is read (self-adjoint view),
//     stop when |r|^2 < max(tol^2 |b|^2, DBL_MIN) or after maxIterations (default 2n).
//   * Transform::computeRotationScaling (Fem3DElementCorotationalTetrahedron.cpp:154): SVD
//     F = U diag(s) V^T with s sorted decreasingly, x = det(U V^T) = +-1 applied to the
//     smallest singular value: R = U diag(1,1,x) V^T, S = V diag(s0,s1,x s2) V^T.
//   * computeInverseAndDetWithCheck (…CorotationalTetrahedron.cpp:65,210): invertible iff
//     |det| > 1e-12 (Eigen's dummy_precision for double).
//
// Build: oracle/Makefile (g++ -O3 -ffp-contract=off, so x86-64 and aarch64 give identical bits).

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cfloat>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>

namespace {

using std::vector;

constexpr double kDummyPrecision = 1e-12;

enum Status { ORC_OK = 0, ORC_INVALID_ARG = 1, ORC_DEGENERATE = 2, ORC_CG_MAXITER = 3, ORC_NONFINITE = 4 };

// Fem3DElementTetrahedron.cpp:34-38 (same term order).
double det3v(const double* a, const double* b, const double* c)
{
	return a[0] * b[1] * c[2] + a[2] * b[0] * c[1] + a[1] * b[2] * c[0] - a[2] * b[1] * c[0] - a[1] * b[0] * c[2] -
		   a[0] * b[2] * c[1];
}

double det33(const double m[3][3])
{
	return m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
		   m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
}

// 3x3 inverse by adjugate; returns false when |det| <= 1e-12 (computeInverseAndDetWithCheck).
bool inverse33(const double m[3][3], double inv[3][3])
{
	double d = det33(m);
	if (!(std::abs(d) > kDummyPrecision)) return false;
	double id = 1.0 / d;
	inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
	inv[0][1] = (m[0][2] * m[2][1] - m[0][1] * m[2][2]) * id;
	inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
	inv[1][0] = (m[1][2] * m[2][0] - m[1][0] * m[2][2]) * id;
	inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
	inv[1][2] = (m[0][2] * m[1][0] - m[0][0] * m[1][2]) * id;
	inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
	inv[2][1] = (m[0][1] * m[2][0] - m[0][0] * m[2][1]) * id;
	inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
	return true;
}

// 4x4 inverse by cofactor expansion; returns false when |det| <= 1e-12.
bool inverse44(const double a[4][4], double inv[4][4])
{
	double cof[4][4];
	for (int i = 0; i < 4; ++i)
	{
		for (int j = 0; j < 4; ++j)
		{
			double m[3][3];
			int r = 0;
			for (int ii = 0; ii < 4; ++ii)
			{
				if (ii == i) continue;
				int c = 0;
				for (int jj = 0; jj < 4; ++jj)
				{
					if (jj == j) continue;
					m[r][c++] = a[ii][jj];
				}
				++r;
			}
			double s = ((i + j) % 2 == 0) ? 1.0 : -1.0;
			cof[i][j] = s * det33(m);
		}
	}
	double d = 0.0;
	for (int j = 0; j < 4; ++j) d += a[0][j] * cof[0][j];
	if (!(std::abs(d) > kDummyPrecision)) return false;
	for (int i = 0; i < 4; ++i)
		for (int j = 0; j < 4; ++j) inv[i][j] = cof[j][i] / d;
	return true;
}

// One-sided (Hestenes) Jacobi SVD of a 3x3 matrix: F = U diag(s) V^T, s sorted decreasingly.
void svd33(const double F[3][3], double U[3][3], double s[3], double V[3][3])
{
	double A[3][3];
	std::memcpy(A, F, sizeof(A));
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
	const int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
	for (int sweep = 0; sweep < 60; ++sweep)
	{
		bool rotated = false;
		for (auto& pq : pairs)
		{
			int p = pq[0], q = pq[1];
			double alpha = 0, beta = 0, gamma = 0;
			for (int k = 0; k < 3; ++k)
			{
				alpha += A[k][p] * A[k][p];
				beta += A[k][q] * A[k][q];
				gamma += A[k][p] * A[k][q];
			}
			if (gamma == 0.0 || std::abs(gamma) <= DBL_EPSILON * std::sqrt(alpha * beta)) continue;
			rotated = true;
			double zeta = (beta - alpha) / (2.0 * gamma);
			double t = (zeta >= 0 ? 1.0 : -1.0) / (std::abs(zeta) + std::sqrt(1.0 + zeta * zeta));
			double c = 1.0 / std::sqrt(1.0 + t * t);
			double sn = c * t;
			for (int k = 0; k < 3; ++k)
			{
				double ap = A[k][p], aq = A[k][q];
				A[k][p] = c * ap - sn * aq;
				A[k][q] = sn * ap + c * aq;
				double vp = V[k][p], vq = V[k][q];
				V[k][p] = c * vp - sn * vq;
				V[k][q] = sn * vp + c * vq;
			}
		}
		if (!rotated) break;
	}
	double sv[3];
	for (int j = 0; j < 3; ++j) sv[j] = std::sqrt(A[0][j] * A[0][j] + A[1][j] * A[1][j] + A[2][j] * A[2][j]);
	int order[3] = {0, 1, 2};
	std::sort(order, order + 3, [&](int a, int b) { return sv[a] > sv[b]; });
	double A2[3][3], V2[3][3];
	for (int j = 0; j < 3; ++j)
	{
		s[j] = sv[order[j]];
		for (int k = 0; k < 3; ++k)
		{
			A2[k][j] = A[k][order[j]];
			V2[k][j] = V[k][order[j]];
		}
	}
	std::memcpy(V, V2, sizeof(V2));
	// U columns: normalised columns of A; rank-deficient columns are completed orthonormally.
	for (int j = 0; j < 3; ++j)
	{
		if (s[j] > 1e-12 * std::max(s[0], 1e-300) && s[j] > 0)
		{
			for (int k = 0; k < 3; ++k) U[k][j] = A2[k][j] / s[j];
		}
		else if (j == 2)
		{
			U[0][2] = U[1][0] * U[2][1] - U[2][0] * U[1][1];
			U[1][2] = U[2][0] * U[0][1] - U[0][0] * U[2][1];
			U[2][2] = U[0][0] * U[1][1] - U[1][0] * U[0][1];
		}
		else
		{
			// Pick the canonical axis least aligned with the previous columns and orthonormalise.
			double best[3] = {1, 0, 0};
			double bestDot = 2.0;
			for (int ax = 0; ax < 3; ++ax)
			{
				double d = 0;
				for (int jj = 0; jj < j; ++jj) d += std::abs(U[ax][jj]);
				if (d < bestDot)
				{
					bestDot = d;
					best[0] = best[1] = best[2] = 0;
					best[ax] = 1;
				}
			}
			for (int jj = 0; jj < j; ++jj)
			{
				double d = best[0] * U[0][jj] + best[1] * U[1][jj] + best[2] * U[2][jj];
				for (int k = 0; k < 3; ++k) best[k] -= d * U[k][jj];
			}
			double nrm = std::sqrt(best[0] * best[0] + best[1] * best[1] + best[2] * best[2]);
			for (int k = 0; k < 3; ++k) U[k][j] = best[k] / nrm;
		}
	}
}

// Transform::computeRotationScaling restated (see file header): F = R S.
void polar33(const double F[3][3], double R[3][3], double S[3][3])
{
	double U[3][3], s[3], V[3][3];
	svd33(F, U, s, V);
	double x = (det33(U) * det33(V) < 0.0) ? -1.0 : 1.0;
	double sv[3] = {s[0], s[1], s[2] * x};
	for (int i = 0; i < 3; ++i)
	{
		for (int j = 0; j < 3; ++j)
		{
			double r = 0, sc = 0;
			for (int k = 0; k < 3; ++k)
			{
				double uk = (k == 2) ? U[i][k] * x : U[i][k];
				r += uk * V[j][k];
				sc += V[i][k] * sv[k] * V[j][k];
			}
			R[i][j] = r;
			S[i][j] = sc;
		}
	}
}

// ---------------------------------------------------------------------------------------------
// Element: Fem3DElementTetrahedron (rest precompute) + Fem3DElementCorotationalTetrahedron.
// ---------------------------------------------------------------------------------------------
struct Tet
{
	int n[4];
	double E, nu, rho;
	double x0[12];
	double Vinv[4][4];
	double M0[12][12], K0[12][12];
	double R[3][3];
	double M[12][12], K[12][12];
	double f[12];
	bool orientationWarning = false;
	bool linear = false;   // Fem3DElementTetrahedron instead of the corotational element
	int singularG = 0;     // count of updates that hit the singular-G early return
	int invalidRotation = 0;  // count of updates that hit the |det R - 1| > 1e-8 early return
};

// Fem3DElementTetrahedron::getVolume, Fem3DElementTetrahedron.cpp:218-235.
double tetVolume(const double* p0, const double* p1, const double* p2, const double* p3)
{
	return (det3v(p1, p2, p3) - det3v(p0, p2, p3) + det3v(p0, p1, p3) - det3v(p0, p1, p2)) / 6.0;
}

// Fem3DElementCorotationalTetrahedron::computeRotationMassAndStiffness,
// Fem3DElementCorotationalTetrahedron.cpp:116-288 (Me/Ke pointers both set, as for FMDK).
void computeRotationMassAndStiffness(Tet& t, const double* x /*12*/, bool wantM, bool wantK)
{
	// F = P.V^-1 (:136-146); only the linear 3x3 part enters the polar decomposition.
	double P[4][4];
	for (int a = 0; a < 4; ++a)
	{
		for (int k = 0; k < 3; ++k) P[k][a] = x[3 * a + k];
		P[3][a] = 1.0;
	}
	double F[3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			double s = 0;
			for (int k = 0; k < 4; ++k) s += P[i][k] * t.Vinv[k][j];
			F[i][j] = s;
		}
	double R[3][3], S[3][3];
	polar33(F, R, S);  // :154
	std::memcpy(t.R, R, sizeof(R));  // :156-159
	if (std::abs(det33(R) - 1.0) > 1e-8)  // :161-166 (a NaN rotation passes, as in the reference)
	{
		t.invalidRotation++;
		return;
	}
	double R12[12][12] = {};
	for (int b = 0; b < 4; ++b)
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j) R12[3 * b + i][3 * b + j] = R[i][j];  // :173-178

	auto mul12 = [](const double A[12][12], const double B[12][12], double C[12][12], bool transB) {
		for (int i = 0; i < 12; ++i)
			for (int j = 0; j < 12; ++j)
			{
				double s = 0;
				for (int k = 0; k < 12; ++k) s += A[i][k] * (transB ? B[j][k] : B[k][j]);
				C[i][j] = s;
			}
	};
	if (wantM)  // :182-186
	{
		double RM[12][12];
		mul12(R12, t.M0, RM, false);
		mul12(RM, R12, t.M, true);
	}
	if (!wantK) return;
	double RK[12][12];
	mul12(R12, t.K0, RK, false);  // :202
	mul12(RK, R12, t.K, true);    // :203 (m_K now holds R.K0.R^t)

	double trS = S[0][0] + S[1][1] + S[2][2];
	double G[3][3], Ginv[3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			double s = 0;
			for (int k = 0; k < 3; ++k) s += ((i == k ? trS : 0.0) - S[i][k]) * R[j][k];
			G[i][j] = s;  // :208
		}
	if (!inverse33(G, Ginv))  // :210-216
	{
		t.singularG++;
		return;
	}
	// dR/dF_ij = [w_ij] R with w_ij = Ginv * 2 * skew(R^T e_i e_j^T) (:220-233).
	double dRdF[3][3][3][3];
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j)
		{
			// R^T e_i e_j^T has column j equal to row i of R, zeros elsewhere.
			double A[3][3] = {};
			for (int k = 0; k < 3; ++k) A[k][j] = R[i][k];
			double sk[3] = {(A[2][1] - A[1][2]) / 2.0, (A[0][2] - A[2][0]) / 2.0, (A[1][0] - A[0][1]) / 2.0};
			double w[3];
			for (int k = 0; k < 3; ++k) w[k] = (Ginv[k][0] * 2.0) * sk[0] + (Ginv[k][1] * 2.0) * sk[1] + (Ginv[k][2] * 2.0) * sk[2];
			double W[3][3] = {{0, -w[2], w[1]}, {w[2], 0, -w[0]}, {-w[1], w[0], 0}};
			for (int r = 0; r < 3; ++r)
				for (int c = 0; c < 3; ++c)
				{
					double s = 0;
					for (int k = 0; k < 3; ++k) s += W[r][k] * R[k][c];
					dRdF[i][j][r][c] = s;
				}
		}
	// dR/dx_l (:251-269): dRdX[l](i,j) = dRdF[i][j].row(axis) . n_node, n_node = V^-1 row, first 3.
	double dRdX[12][3][3];
	for (int node = 0; node < 4; ++node)
		for (int axis = 0; axis < 3; ++axis)
		{
			int l = 3 * node + axis;
			for (int i = 0; i < 3; ++i)
				for (int j = 0; j < 3; ++j)
				{
					double s = 0;
					for (int k = 0; k < 3; ++k) s += dRdF[i][j][axis][k] * t.Vinv[node][k];
					dRdX[l][i][j] = s;
				}
		}
	// KTimesRx_x0 = m_K (R12^T x - x0), with m_K already R.K0.R^t (:276).
	double Rtx_x0[12], KTx[12];
	for (int i = 0; i < 12; ++i)
	{
		double s = 0;
		for (int k = 0; k < 12; ++k) s += R12[k][i] * x[k];
		Rtx_x0[i] = s - t.x0[i];
	}
	for (int i = 0; i < 12; ++i)
	{
		double s = 0;
		for (int k = 0; k < 12; ++k) s += t.K[i][k] * Rtx_x0[k];
		KTx[i] = s;
	}
	// K.col(l) += dRdxl12 * KTimesRx_x0 + (RK * dRdxl12^T) * x (:277-286).
	for (int l = 0; l < 12; ++l)
	{
		double D12[12][12] = {};
		for (int b = 0; b < 4; ++b)
			for (int i = 0; i < 3; ++i)
				for (int j = 0; j < 3; ++j) D12[3 * b + i][3 * b + j] = dRdX[l][i][j];
		double RKDt[12][12];
		mul12(RK, D12, RKDt, true);
		for (int i = 0; i < 12; ++i)
		{
			double s1 = 0, s2 = 0;
			for (int k = 0; k < 12; ++k)
			{
				s1 += D12[i][k] * KTx[k];
				s2 += RKDt[i][k] * x[k];
			}
			t.K[i][l] += s1 + s2;
		}
	}
}

// Fem3DElementCorotationalTetrahedron::doUpdateFMDK, :77-114 (options = FMDK); with `linear`,
// Fem3DElementTetrahedron::doUpdateFMDK (Fem3DElementTetrahedron.cpp:77-90): M = M0, K = K0,
// f = -K0 (x - x0).
void tetUpdateFMDK(Tet& t, const double* X /*global positions*/)
{
	const bool linear = t.linear;
	double x[12];
	for (int a = 0; a < 4; ++a)
		for (int k = 0; k < 3; ++k) x[3 * a + k] = X[3 * t.n[a] + k];
	if (linear)
	{
		for (int i = 0; i < 12; ++i)
			for (int j = 0; j < 12; ++j)
			{
				t.M[i][j] = t.M0[i][j];
				t.K[i][j] = t.K0[i][j];
			}
		for (int i = 0; i < 3; ++i)
			for (int j = 0; j < 3; ++j) t.R[i][j] = (i == j) ? 1.0 : 0.0;
		for (int i = 0; i < 12; ++i)
		{
			double s = 0;
			for (int k = 0; k < 12; ++k) s += t.K0[i][k] * (x[k] - t.x0[k]);
			t.f[i] = -s;
		}
		return;
	}
	computeRotationMassAndStiffness(t, x, true, true);
	double Rx0[12];
	for (int a = 0; a < 4; ++a)
		for (int i = 0; i < 3; ++i)
		{
			double s = 0;
			for (int k = 0; k < 3; ++k) s += t.R[i][k] * t.x0[3 * a + k];
			Rx0[3 * a + i] = s;
		}
	for (int i = 0; i < 12; ++i)
	{
		double s = 0;
		for (int k = 0; k < 12; ++k) s += t.K[i][k] * (x[k] - Rx0[k]);
		t.f[i] = -s;
	}
}

// Fem3DElementTetrahedron::initialize + computeMass + computeStiffness + computeShapeFunctions
// (Fem3DElementTetrahedron.cpp:92-216, 237-359), then Fem3DElementCorotationalTetrahedron::initialize
// (Fem3DElementCorotationalTetrahedron.cpp:48-75). Returns ORC_DEGENERATE when V is not invertible.
int tetInitialize(Tet& t, const double* X)
{
	// FemElement::initialize material checks, FemElement.cpp:33-43.
	if (!(t.rho > 0.0) || !(t.nu > 0.0 && t.nu < 0.5) || !(t.E > 0.0)) return ORC_INVALID_ARG;
	for (int a = 0; a < 4; ++a)
		for (int k = 0; k < 3; ++k) t.x0[3 * a + k] = X[3 * t.n[a] + k];
	const double *A = t.x0, *B = t.x0 + 3, *C = t.x0 + 6, *D = t.x0 + 9;
	double AB[3], AC[3], AD[3];
	for (int k = 0; k < 3; ++k)
	{
		AB[k] = B[k] - A[k];
		AC[k] = C[k] - A[k];
		AD[k] = D[k] - A[k];
	}
	double cr[3] = {AB[1] * AC[2] - AB[2] * AC[1], AB[2] * AC[0] - AB[0] * AC[2], AB[0] * AC[1] - AB[1] * AC[0]};
	t.orientationWarning = (cr[0] * AD[0] + cr[1] * AD[1] + cr[2] * AD[2]) < 0;  // :106-116

	double vol = tetVolume(A, B, C, D);
	// computeMass (:149-165)
	double coef = vol * t.rho / 20.0;
	for (int i = 0; i < 12; ++i)
		for (int j = 0; j < 12; ++j)
			t.M0[i][j] = ((i % 3) == (j % 3)) ? ((i / 3 == j / 3) ? 2.0 * coef : coef) : 0.0;
	// computeShapeFunctions (:274-357)
	double ai[4], bi[4], ci[4], di[4];
	ai[0] = det3v(B, C, D);
	ai[1] = -det3v(A, C, D);
	ai[2] = det3v(A, B, D);
	ai[3] = -det3v(A, B, C);
	{
		double at[3] = {1, A[1], A[2]}, bt[3] = {1, B[1], B[2]}, ct[3] = {1, C[1], C[2]}, dt[3] = {1, D[1], D[2]};
		bi[0] = -det3v(bt, ct, dt);
		bi[1] = det3v(at, ct, dt);
		bi[2] = -det3v(at, bt, dt);
		bi[3] = det3v(at, bt, ct);
	}
	{
		double at[3] = {1, A[0], A[2]}, bt[3] = {1, B[0], B[2]}, ct[3] = {1, C[0], C[2]}, dt[3] = {1, D[0], D[2]};
		ci[0] = det3v(bt, ct, dt);
		ci[1] = -det3v(at, ct, dt);
		ci[2] = det3v(at, bt, dt);
		ci[3] = -det3v(at, bt, ct);
	}
	{
		double at[3] = {1, A[0], A[1]}, bt[3] = {1, B[0], B[1]}, ct[3] = {1, C[0], C[1]}, dt[3] = {1, D[0], D[1]};
		di[0] = -det3v(bt, ct, dt);
		di[1] = det3v(at, ct, dt);
		di[2] = -det3v(at, bt, dt);
		di[3] = det3v(at, bt, ct);
	}
	(void)ai;
	// computeStiffness (:172-215)
	double Bm[6][12] = {};
	double c6 = 1.0 / (6.0 * vol);
	for (int i = 0; i < 4; ++i)
	{
		Bm[0][3 * i] = c6 * bi[i];
		Bm[1][3 * i + 1] = c6 * ci[i];
		Bm[2][3 * i + 2] = c6 * di[i];
		Bm[3][3 * i] = c6 * ci[i];
		Bm[3][3 * i + 1] = c6 * bi[i];
		Bm[4][3 * i + 1] = c6 * di[i];
		Bm[4][3 * i + 2] = c6 * ci[i];
		Bm[5][3 * i] = c6 * di[i];
		Bm[5][3 * i + 2] = c6 * bi[i];
	}
	double lambda = t.E * t.nu / ((1.0 + t.nu) * (1.0 - 2.0 * t.nu));
	double mu = t.E / (2.0 * (1 + t.nu));
	double Em[6][6] = {};
	Em[0][0] = Em[1][1] = Em[2][2] = 2.0 * mu + lambda;
	Em[0][1] = Em[0][2] = Em[1][0] = Em[1][2] = Em[2][0] = Em[2][1] = lambda;
	Em[3][3] = Em[4][4] = Em[5][5] = mu;
	double EB[6][12];
	for (int i = 0; i < 6; ++i)
		for (int j = 0; j < 12; ++j)
		{
			double s = 0;
			for (int k = 0; k < 6; ++k) s += Em[i][k] * Bm[k][j];
			EB[i][j] = s;
		}
	double K[12][12];
	for (int i = 0; i < 12; ++i)
		for (int j = 0; j < 12; ++j)
		{
			double s = 0;
			for (int k = 0; k < 6; ++k) s += Bm[k][i] * EB[k][j];
			K[i][j] = vol * s;
		}
	for (int i = 0; i < 12; ++i)
		for (int j = 0; j < 12; ++j) t.K0[i][j] = (K[i][j] + K[j][i]) * 0.5;

	// Corotational initialize: m_MLinear/m_KLinear, V^-1 (:53-72).
	double V[4][4];
	for (int a = 0; a < 4; ++a)
	{
		for (int k = 0; k < 3; ++k) V[k][a] = t.x0[3 * a + k];
		V[3][a] = 1.0;
	}
	if (!inverse44(V, t.Vinv)) return ORC_DEGENERATE;
	std::memcpy(t.M, t.M0, sizeof(t.M));
	std::memcpy(t.K, t.K0, sizeof(t.K));
	for (int i = 0; i < 3; ++i)
		for (int j = 0; j < 3; ++j) t.R[i][j] = (i == j);
	tetUpdateFMDK(t, X);  // :74
	return ORC_OK;
}

// ---------------------------------------------------------------------------------------------
// Element: Fem3DElementCube (trilinear hexahedron, 2x2x2 Gauss-Legendre quadrature). A linear
// element: K and M are computed once at the rest state, f = -K (x - x0) (:129-141).
// ---------------------------------------------------------------------------------------------
struct Hex
{
	int n[8];
	double E, nu, rho;
	double x0[24];
	double K0[24][24], M0[24][24];
	double f[24];
	double volume = 0.0;
};

// Shape-function signs of the 8 corners (Fem3DElementCube.cpp:72-74).
const double kHexSignEps[8] = {-1.0, +1.0, +1.0, -1.0, -1.0, +1.0, +1.0, -1.0};
const double kHexSignEta[8] = {-1.0, -1.0, +1.0, +1.0, -1.0, -1.0, +1.0, +1.0};
const double kHexSignMu[8] = {-1.0, -1.0, -1.0, -1.0, +1.0, +1.0, +1.0, +1.0};

// gaussQuadrature2Points (GaussLegendreQuadrature.cpp:30-34): +1/sqrt(3) then -1/sqrt(3), weight 1.
double gaussPoint2(int i) { return (i == 0 ? 1.0 : -1.0) / std::sqrt(3.0); }

// shapeFunction and its derivatives (Fem3DElementCube.cpp:368-398).
double hexN(int i, double e, double h, double m)
{
	return 1.0 / 8.0 * (1 + e * kHexSignEps[i]) * (1 + h * kHexSignEta[i]) * (1 + m * kHexSignMu[i]);
}
double hexdNde(int i, double, double h, double m)
{
	return 1.0 / 8.0 * kHexSignEps[i] * (1 + h * kHexSignEta[i]) * (1 + m * kHexSignMu[i]);
}
double hexdNdh(int i, double e, double, double m)
{
	return 1.0 / 8.0 * (1 + e * kHexSignEps[i]) * kHexSignEta[i] * (1 + m * kHexSignMu[i]);
}
double hexdNdm(int i, double e, double h, double)
{
	return 1.0 / 8.0 * (1 + e * kHexSignEps[i]) * (1 + h * kHexSignEta[i]) * kHexSignMu[i];
}

// evaluateJ (Fem3DElementCube.cpp:169-211): J(r, axis) = sum_i p_i[axis] dN_i/d(eps, eta, mu)_r.
// Returns false when J is not invertible (|det J| <= 1e-12, the SURGSIM_ASSERT of :202-207).
bool hexJacobian(const double* p /*24*/, double e, double h, double m, double Jinv[3][3], double* detJ)
{
	double J[3][3] = {};
	for (int i = 0; i < 8; ++i)
		for (int axis = 0; axis < 3; ++axis)
		{
			J[0][axis] += p[3 * i + axis] * hexdNde(i, e, h, m);
			J[1][axis] += p[3 * i + axis] * hexdNdh(i, e, h, m);
			J[2][axis] += p[3 * i + axis] * hexdNdm(i, e, h, m);
		}
	*detJ = det33(J);
	return inverse33(J, Jinv);
}

// getVolume (Fem3DElementCube.cpp:321-366): sum of w_i w_j w_k det J over the 8 Gauss points.
// Returns ORC_DEGENERATE when a Jacobian is singular or the volume is not above 1e-12 (:357).
int hexVolume(const double* p, double* vol)
{
	double v = 0.0;
	for (int i = 0; i < 2; ++i)
		for (int j = 0; j < 2; ++j)
			for (int k = 0; k < 2; ++k)
			{
				double Jinv[3][3], detJ;
				if (!hexJacobian(p, gaussPoint2(i), gaussPoint2(j), gaussPoint2(k), Jinv, &detJ)) return ORC_DEGENERATE;
				v += 1.0 * 1.0 * 1.0 * detJ;
			}
	*vol = v;
	return v > 1e-12 ? ORC_OK : ORC_DEGENERATE;
}

// Fem3DElementCube::initialize (Fem3DElementCube.cpp:65-95): material checks, rest positions, rest
// volume, then computeMass (:97-127, addMassMatrixAtPoint :290-319) and computeStiffness (:143-167,
// evaluateStrainDisplacement :213-251, buildConstitutiveMaterialMatrix :253-265,
// addStrainStressStiffnessAtPoint :267-288).
int hexInitialize(Hex& t, const double* X)
{
	if (!(t.rho > 0.0) || !(t.nu > 0.0 && t.nu < 0.5) || !(t.E > 0.0)) return ORC_INVALID_ARG;
	for (int a = 0; a < 8; ++a)
		for (int k = 0; k < 3; ++k) t.x0[3 * a + k] = X[3 * (size_t)t.n[a] + k];
	int st = hexVolume(t.x0, &t.volume);
	if (st != ORC_OK) return st;
	const double lambda = t.E * t.nu / ((1.0 + t.nu) * (1.0 - 2.0 * t.nu));
	const double mu = t.E / (2.0 * (1 + t.nu));
	double C[6][6] = {};
	C[0][0] = C[1][1] = C[2][2] = 2.0 * mu + lambda;
	C[0][1] = C[0][2] = C[1][0] = C[1][2] = C[2][0] = C[2][1] = lambda;
	C[3][3] = C[4][4] = C[5][5] = mu;
	std::memset(t.M0, 0, sizeof(t.M0));
	std::memset(t.K0, 0, sizeof(t.K0));
	for (int gi = 0; gi < 2; ++gi)
		for (int gj = 0; gj < 2; ++gj)
			for (int gk = 0; gk < 2; ++gk)
			{
				const double e = gaussPoint2(gi), h = gaussPoint2(gj), m = gaussPoint2(gk);
				double Jinv[3][3], detJ;
				if (!hexJacobian(t.x0, e, h, m, Jinv, &detJ)) return ORC_DEGENERATE;
				const double w = 1.0 * 1.0 * 1.0 * detJ;
				// M += w rho phi^T phi, phi = (N_i I3) side by side.
				double N[8];
				for (int i = 0; i < 8; ++i) N[i] = hexN(i, e, h, m);
				for (int a = 0; a < 8; ++a)
					for (int b = 0; b < 8; ++b)
						for (int k = 0; k < 3; ++k) t.M0[3 * a + k][3 * b + k] += (w * t.rho) * (N[a] * N[b]);
				// B (6x24): dN_i/d(x,y,z) = J^-1 dN_i/d(eps,eta,mu), Voigt rows xx yy zz xy yz zx.
				double B[6][24] = {};
				for (int i = 0; i < 8; ++i)
				{
					const double dl[3] = {hexdNde(i, e, h, m), hexdNdh(i, e, h, m), hexdNdm(i, e, h, m)};
					double g[3];
					for (int r = 0; r < 3; ++r) g[r] = Jinv[r][0] * dl[0] + Jinv[r][1] * dl[1] + Jinv[r][2] * dl[2];
					B[0][3 * i] = g[0];
					B[1][3 * i + 1] = g[1];
					B[2][3 * i + 2] = g[2];
					B[3][3 * i] = g[1];
					B[3][3 * i + 1] = g[0];
					B[4][3 * i + 1] = g[2];
					B[4][3 * i + 2] = g[1];
					B[5][3 * i] = g[2];
					B[5][3 * i + 2] = g[0];
				}
				// K += (w B^T) C B, evaluated left to right.
				double BtC[24][6];
				for (int r = 0; r < 24; ++r)
					for (int c = 0; c < 6; ++c)
					{
						double s = 0;
						for (int l = 0; l < 6; ++l) s += (w * B[l][r]) * C[l][c];
						BtC[r][c] = s;
					}
				for (int r = 0; r < 24; ++r)
					for (int c = 0; c < 24; ++c)
					{
						double s = 0;
						for (int l = 0; l < 6; ++l) s += BtC[r][l] * B[l][c];
						t.K0[r][c] += s;
					}
			}
	return ORC_OK;
}

// doUpdateFMDK (Fem3DElementCube.cpp:129-141): f = -K (x - x0); M and K stay the rest matrices.
void hexUpdateF(Hex& t, const double* X)
{
	double u[24];
	for (int a = 0; a < 8; ++a)
		for (int k = 0; k < 3; ++k) u[3 * a + k] = X[3 * (size_t)t.n[a] + k] - t.x0[3 * a + k];
	for (int r = 0; r < 24; ++r)
	{
		double s = 0;
		for (int c = 0; c < 24; ++c) s += t.K0[r][c] * u[c];
		t.f[r] = -s;
	}
}

// ---------------------------------------------------------------------------------------------
// CSC matrix helpers (Eigen::SparseMatrix<double, ColMajor, int> semantics).
// ---------------------------------------------------------------------------------------------
struct Pattern
{
	int n = 0;
	vector<int> colptr, rowidx;
	int64_t nnz() const { return (int64_t)rowidx.size(); }
	// Position of (row, col), or -1 (binary search like SparseCompressedBase::searchLowerIndex).
	int64_t find(int row, int col) const
	{
		auto b = rowidx.begin() + colptr[col], e = rowidx.begin() + colptr[col + 1];
		auto it = std::lower_bound(b, e, row);
		if (it == e || *it != row) return -1;
		return it - rowidx.begin();
	}
};

// y = A x (column-major sparse * dense, Eigen's sparse_time_dense_product order).
void spmv(const Pattern& p, const double* vals, const double* x, double* y)
{
	std::fill(y, y + p.n, 0.0);
	for (int j = 0; j < p.n; ++j)
	{
		double xj = x[j];
		for (int k = p.colptr[j]; k < p.colptr[j + 1]; ++k) y[p.rowidx[k]] += vals[k] * xj;
	}
}

// y = selfadjointView<Lower>(A) x: entries with row >= col are used, mirrored to the upper part.
void spmvLowerSym(const Pattern& p, const double* vals, const double* x, double* y)
{
	std::fill(y, y + p.n, 0.0);
	for (int j = 0; j < p.n; ++j)
	{
		double xj = x[j];
		double resj = 0.0;
		for (int k = p.colptr[j]; k < p.colptr[j + 1]; ++k)
		{
			int i = p.rowidx[k];
			if (i < j) continue;
			if (i == j)
			{
				y[j] += vals[k] * xj;
				continue;
			}
			y[i] += vals[k] * xj;
			resj += vals[k] * x[i];
		}
		y[j] += resj;
	}
}

struct CgResult
{
	int iterations = 0;
	double error = 0.0;
	bool converged = true;
};

// Eigen::ConjugateGradient<…, Lower, DiagonalPreconditioner>::solve with x0 = 0,
// as called by LinearSparseSolveAndInverseCG::solve (LinearSparseSolveAndInverse.cpp:126-129).
CgResult cgSolve(const Pattern& p, const double* vals, const double* b, double* x, double tol, int maxIter)
{
	const int n = p.n;
	CgResult res;
	if (maxIter < 0) maxIter = 2 * n;
	// DiagonalPreconditioner::factorize: 1/diag, or 1 where the diagonal is missing or zero.
	vector<double> invdiag(n, 1.0);
	for (int j = 0; j < n; ++j)
	{
		int64_t k = p.find(j, j);
		if (k >= 0 && vals[k] != 0.0) invdiag[j] = 1.0 / vals[k];
	}
	std::fill(x, x + n, 0.0);
	vector<double> r(b, b + n), z(n), pdir(n), tmp(n);
	double rhsNorm2 = 0;
	for (int i = 0; i < n; ++i) rhsNorm2 += b[i] * b[i];
	if (rhsNorm2 == 0)
	{
		res.iterations = 0;
		res.error = 0;
		return res;
	}
	const double threshold = std::max(tol * tol * rhsNorm2, DBL_MIN);
	double residualNorm2 = rhsNorm2;  // residual = b - A*0
	if (residualNorm2 < threshold)
	{
		res.error = std::sqrt(residualNorm2 / rhsNorm2);
		return res;
	}
	for (int i = 0; i < n; ++i) pdir[i] = invdiag[i] * r[i];
	double absNew = 0;
	for (int i = 0; i < n; ++i) absNew += r[i] * pdir[i];
	int it = 0;
	while (it < maxIter)
	{
		spmvLowerSym(p, vals, pdir.data(), tmp.data());
		double pq = 0;
		for (int i = 0; i < n; ++i) pq += pdir[i] * tmp[i];
		double alpha = absNew / pq;
		for (int i = 0; i < n; ++i) x[i] += alpha * pdir[i];
		for (int i = 0; i < n; ++i) r[i] -= alpha * tmp[i];
		residualNorm2 = 0;
		for (int i = 0; i < n; ++i) residualNorm2 += r[i] * r[i];
		if (residualNorm2 < threshold) break;
		for (int i = 0; i < n; ++i) z[i] = invdiag[i] * r[i];
		double absOld = absNew;
		absNew = 0;
		for (int i = 0; i < n; ++i) absNew += r[i] * z[i];
		double beta = absNew / absOld;
		for (int i = 0; i < n; ++i) pdir[i] = z[i] + beta * pdir[i];
		++it;
	}
	res.iterations = it;
	res.error = std::sqrt(residualNorm2 / rhsNorm2);
	res.converged = residualNorm2 < threshold;
	return res;
}

// ---------------------------------------------------------------------------------------------
// OdeEquation / OdeSolverEulerImplicit restated over a generic equation.
// ---------------------------------------------------------------------------------------------
struct Equation
{
	Pattern pat;
	vector<double> M, D, K, f;  // values on pat; f has n entries
	vector<int> bcDofs;          // OdeState boundary conditions (insertion order)
	virtual void updateFMDK(const double* x, const double* v) = 0;
	virtual ~Equation() = default;
};

struct SolverParams
{
	int newtonMaxIter = 1;        // OdeSolverEulerImplicit.cpp:26
	double newtonEps = 1e-5;      // :26
	double cgTol = DBL_EPSILON;   // Eigen default tolerance
	int cgMaxIter = -1;           // Eigen default 2n
};

struct StepStats
{
	int cgIterations = 0;  // summed over Newton iterations
	double cgError = 0;
	bool cgConverged = true;
	int newtonIterations = 0;
	double tElement = 0, tAssemble = 0, tSystem = 0, tSolve = 0;
};

double nowSec()
{
	return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// OdeSolverEulerImplicit::solve(dt, cur, new, computeCompliance=false), OdeSolverEulerImplicit.cpp:55-122,
// with assembleLinearSystem :124-161. xn/vn receive the new state.
struct ImplicitEuler
{
	SolverParams prm;
	vector<double> S, rhs, solution, prevSolution;
	StepStats stats;

	void assemble(Equation& eq, double dt, const double* xt, const double* vt, const double* xn, const double* vn)
	{
		double t0 = nowSec();
		eq.updateFMDK(xn, vn);  // :140
		double t1 = nowSec();
		const int64_t nnz = eq.pat.nnz();
		const int n = eq.pat.n;
		S.resize(nnz);
		for (int64_t k = 0; k < nnz; ++k) S[k] = eq.M[k] * (1.0 / dt) + eq.D[k] + eq.K[k] * dt;  // :148
		// OdeState::applyBoundaryConditionsToMatrix(SparseMatrix*, true), OdeState.cpp:197-218.
		for (int d : eq.bcDofs)
		{
			// zeroRow (SparseMatrix.h:352-362) visits every column; the pattern is structurally
			// symmetric, so the columns holding row d are exactly the rows of column d.
			for (int64_t kk = eq.pat.colptr[d]; kk < eq.pat.colptr[d + 1]; ++kk)
			{
				int64_t k = eq.pat.find(d, eq.pat.rowidx[kk]);
				if (k >= 0 && S[k] != 0.0) S[k] = 0.0;
			}
			for (int64_t k = eq.pat.colptr[d]; k < eq.pat.colptr[d + 1]; ++k)  // zeroColumn (:368-377)
				if (S[k] != 0.0) S[k] = 0.0;
			int64_t kd = eq.pat.find(d, d);
			if (kd >= 0) S[kd] = 1.0;
		}
		// rhs = f + K (x_n - x_t - v_n dt) - M (v_n - v_t) / dt, BC rows zeroed (:155-160).
		vector<double> tmp(n), Kt(n), Mt(n);
		for (int i = 0; i < n; ++i) tmp[i] = (xn[i] - xt[i]) - vn[i] * dt;
		spmv(eq.pat, eq.K.data(), tmp.data(), Kt.data());
		rhs.resize(n);
		for (int i = 0; i < n; ++i) rhs[i] = eq.f[i] + Kt[i];
		for (int i = 0; i < n; ++i) tmp[i] = vn[i] - vt[i];
		spmv(eq.pat, eq.M.data(), tmp.data(), Mt.data());
		for (int i = 0; i < n; ++i) rhs[i] -= Mt[i] / dt;
		for (int d : eq.bcDofs) rhs[d] = 0.0;
		double t2 = nowSec();
		stats.tElement += t1 - t0;
		stats.tSystem += t2 - t1;
	}

	int solve(Equation& eq, double dt, const double* xt, const double* vt, double* xn, double* vn)
	{
		const int n = eq.pat.n;
		stats = StepStats();
		std::copy(xt, xt + n, xn);  // *newState = currentState (:82)
		std::copy(vt, vt + n, vn);
		if (prm.newtonMaxIter > 1) prevSolution.assign(n, 0.0);
		solution.resize(n);
		int it = 0;
		while (it < prm.newtonMaxIter)
		{
			assemble(eq, dt, xt, vt, xn, vn);
			double t0 = nowSec();
			CgResult cr = cgSolve(eq.pat, S.data(), rhs.data(), solution.data(), prm.cgTol, prm.cgMaxIter);
			stats.tSolve += nowSec() - t0;
			stats.cgIterations += cr.iterations;
			stats.cgError = cr.error;
			stats.cgConverged = stats.cgConverged && cr.converged;
			for (int i = 0; i < n; ++i) vn[i] += solution[i];            // :98
			for (int i = 0; i < n; ++i) xn[i] = xt[i] + dt * vn[i];     // :99
			stats.newtonIterations = it + 1;
			if (prm.newtonMaxIter > 1)  // :101-112
			{
				double var = 0;
				for (int i = 0; i < n; ++i) var = std::max(var, std::abs(solution[i] - prevSolution[i]));
				if (var < prm.newtonEps) break;
				prevSolution = solution;
			}
			++it;
		}
		return ORC_OK;
	}
};

// ---------------------------------------------------------------------------------------------
// FemRepresentation / Fem3DRepresentation with corotational or linear tetrahedra, or hexahedra.
// ---------------------------------------------------------------------------------------------
struct FemModel : Equation
{
	int numNodes = 0;
	vector<double> xrest;
	bool hex = false;     // Fem3DElementCube elements in `hexes` instead of tetrahedra in `tets`
	vector<Tet> tets;
	vector<Hex> hexes;
	vector<double> massPerNode;
	vector<int> scatter;  // per element (3 npe)^2: CSC slot of element entry (3a+i, 3b+j)
	double alpha = 0, beta = 0;          // Rayleigh mass / stiffness coefficients
	bool massLumping = false;            // FemRepresentation::setMassLumping (FemRepresentation.cpp:320-323)
	double gravity[3] = {0.0, -9.81, 0.0};  // Representation.cpp:36
	bool gravityEnabled = true;
	// state (current) and scratch
	vector<double> x, v, xNew, vNew;
	bool active = true;
	ImplicitEuler solver;
	int singularGCount = 0, invalidRotationCount = 0, orientationWarnings = 0;
	// External generalized force, stiffness and damping of the coming update
	// (DeformableRepresentation m_externalGeneralized*), on the pattern; cleared after each step.
	bool hasExternal = false;
	vector<double> fExt, kExt, dExt;

	int nodesPerElement() const { return hex ? 8 : 4; }

	// Fem3DRepresentation::addExternalGeneralizedForce (Fem3DRepresentation.cpp:133-197) with a
	// Fem3DLocalization at element e, natural coordinates coord[npe]: f_ext[node_a] += coord_a F,
	// K_ext / D_ext block (a, b) += coord_a coord_b K / D (K or D may be null).
	int addExternalForce(int e, const double* coord, const double* F, const double* Kx, const double* Dx)
	{
		if (e < 0 || (size_t)e >= numElements() || !coord || !F) return ORC_INVALID_ARG;
		const int npe = nodesPerElement(), Dm = 3 * npe;
		if (!hasExternal)
		{
			fExt.assign(pat.n, 0.0);
			kExt.assign(pat.nnz(), 0.0);
			dExt.assign(pat.nnz(), 0.0);
		}
		const int* nd = elementNodes(e);
		for (int a = 0; a < npe; ++a)
			for (int i = 0; i < 3; ++i) fExt[3 * nd[a] + i] += F[i] * coord[a];
		const int* sm = &scatter[(size_t)e * Dm * Dm];
		for (int a = 0; a < npe; ++a)
			for (int b = 0; b < npe; ++b)
				for (int i = 0; i < 3; ++i)
					for (int j = 0; j < 3; ++j)
					{
						const int k = sm[(3 * a + i) * Dm + 3 * b + j];
						if (Kx) kExt[k] += coord[a] * coord[b] * Kx[3 * i + j];
						if (Dx) dExt[k] += coord[a] * coord[b] * Dx[3 * i + j];
					}
		hasExternal = true;
		return ORC_OK;
	}
	size_t numElements() const { return hex ? hexes.size() : tets.size(); }
	const int* elementNodes(size_t e) const { return hex ? hexes[e].n : tets[e].n; }

	// FemRepresentation::doInitialize (FemRepresentation.cpp:85-132) on the rest state.
	int initialize()
	{
		const int n = 3 * numNodes;
		const int npe = nodesPerElement(), Dm = 3 * npe;
		const size_t E = numElements();
		for (size_t e = 0; e < E; ++e)
			for (int a = 0; a < npe; ++a)
				if (elementNodes(e)[a] < 0 || elementNodes(e)[a] >= numNodes) return ORC_INVALID_ARG;
		for (auto& t : tets)
		{
			int st = tetInitialize(t, xrest.data());
			if (st != ORC_OK) return st;
			orientationWarnings += t.orientationWarning;
		}
		for (auto& t : hexes)
		{
			int st = hexInitialize(t, xrest.data());
			if (st != ORC_OK) return st;
		}
		// massPerNode += getMass / numNodes (:108-117), getMass = volume * rho (FemElement.cpp:105-108).
		massPerNode.assign(numNodes, 0.0);
		for (auto& t : tets)
		{
			double mass = tetVolume(&xrest[3 * t.n[0]], &xrest[3 * t.n[1]], &xrest[3 * t.n[2]], &xrest[3 * t.n[3]]) * t.rho;
			for (int a = 0; a < 4; ++a) massPerNode[t.n[a]] += mass / 4;
		}
		for (auto& t : hexes)
		{
			double mass = t.volume * t.rho;
			for (int a = 0; a < 8; ++a) massPerNode[t.n[a]] += mass / 8;
		}
		// Sparsity: union of the 3x3 node blocks of every element, rows sorted per column (:121-132).
		vector<vector<int>> adj(numNodes);
		for (size_t e = 0; e < E; ++e)
		{
			const int* nd = elementNodes(e);
			for (int a = 0; a < npe; ++a)
				for (int b = 0; b < npe; ++b) adj[nd[b]].push_back(nd[a]);
		}
		for (auto& l : adj)
		{
			std::sort(l.begin(), l.end());
			l.erase(std::unique(l.begin(), l.end()), l.end());
		}
		pat.n = n;
		pat.colptr.assign(n + 1, 0);
		for (int J = 0; J < numNodes; ++J)
			for (int j = 0; j < 3; ++j) pat.colptr[3 * J + j + 1] = 3 * (int)adj[J].size();
		for (int c = 0; c < n; ++c) pat.colptr[c + 1] += pat.colptr[c];
		pat.rowidx.resize(pat.colptr[n]);
		for (int J = 0; J < numNodes; ++J)
			for (int j = 0; j < 3; ++j)
			{
				int k = pat.colptr[3 * J + j];
				for (int I : adj[J])
					for (int i = 0; i < 3; ++i) pat.rowidx[k++] = 3 * I + i;
			}
		// Scatter map: SparseMatrix.h blockWithSearch (:178-242) resolved once per element entry. The
		// first row of block (n_a, n_b) in column 3 n_b + j sits at 3 * (position of n_a in adj[n_b]).
		scatter.resize(E * Dm * Dm);
		for (size_t e = 0; e < E; ++e)
		{
			const int* nd = elementNodes(e);
			for (int b = 0; b < npe; ++b)
			{
				const vector<int>& col = adj[nd[b]];
				for (int a = 0; a < npe; ++a)
				{
					int pos = (int)(std::lower_bound(col.begin(), col.end(), nd[a]) - col.begin());
					for (int j = 0; j < 3; ++j)
					{
						int64_t first = pat.colptr[3 * nd[b] + j] + 3 * pos;
						for (int i = 0; i < 3; ++i)
							scatter[e * Dm * Dm + (3 * a + i) * Dm + 3 * b + j] = (int)(first + i);
					}
				}
			}
		}
		M.assign(pat.nnz(), 0.0);
		D.assign(pat.nnz(), 0.0);
		K.assign(pat.nnz(), 0.0);
		f.assign(n, 0.0);
		x = xrest;
		v.assign(n, 0.0);
		return ORC_OK;
	}

	// FemRepresentation::updateFMDK (:547-563) + OdeEquation::updateFMDK -> computeFMDK (:479-545).
	void updateFMDK(const double* X, const double* V) override
	{
		for (auto& t : tets)
		{
			int sg = t.singularG, ir = t.invalidRotation;
			tetUpdateFMDK(t, X);
			singularGCount += t.singularG - sg;
			invalidRotationCount += t.invalidRotation - ir;
		}
		for (auto& t : hexes) hexUpdateF(t, X);
		const int n = pat.n;
		std::fill(f.begin(), f.end(), 0.0);
		std::fill(M.begin(), M.end(), 0.0);
		std::fill(D.begin(), D.end(), 0.0);
		std::fill(K.begin(), K.end(), 0.0);
		const int npe = nodesPerElement(), Dm = 3 * npe;
		for (size_t e = 0; e < numElements(); ++e)  // FemElement::addFMDK (FemElement.cpp:157-166)
		{
			const int* nd = elementNodes(e);
			const double* fe = hex ? hexes[e].f : tets[e].f;
			const double* Me = hex ? &hexes[e].M0[0][0] : &tets[e].M[0][0];
			const double* Ke = hex ? &hexes[e].K0[0][0] : &tets[e].K[0][0];
			for (int a = 0; a < npe; ++a)
				for (int i = 0; i < 3; ++i) f[3 * nd[a] + i] += fe[3 * a + i];
			const int* s = &scatter[e * Dm * Dm];
			for (int r = 0; r < Dm; ++r)
				for (int c = 0; c < Dm; ++c) M[s[r * Dm + c]] += Me[r * Dm + c];
			for (int r = 0; r < Dm; ++r)
				for (int c = 0; c < Dm; ++c) K[s[r * Dm + c]] += Ke[r * Dm + c];
		}
		const int64_t nnz = pat.nnz();
		if (massLumping)
		{
			// :499-508: for every row, sum = M.row(i).sum() (Eigen walks a column-major row in column
			// order); zeroRow(i) keeps the pattern; M(i, i) = sum.
			vector<double> rowSum(n, 0.0);
			for (int c = 0; c < n; ++c)
				for (int k = pat.colptr[c]; k < pat.colptr[c + 1]; ++k) rowSum[pat.rowidx[k]] += M[k];
			for (int c = 0; c < n; ++c)
				for (int k = pat.colptr[c]; k < pat.colptr[c + 1]; ++k) M[k] = (pat.rowidx[k] == c) ? rowSum[c] : 0.0;
		}
		if (alpha != 0.0)
			for (int64_t k = 0; k < nnz; ++k) D[k] = D[k] + M[k] * alpha;  // :511-514
		if (beta != 0.0)
			for (int64_t k = 0; k < nnz; ++k) D[k] = D[k] + K[k] * beta;  // :515-518
		if (gravityEnabled)  // addGravityForce :641-662
			for (int I = 0; I < numNodes; ++I)
				for (int k = 0; k < 3; ++k) f[3 * I + k] += gravity[k] * (1.0 * massPerNode[I]);
		// addRayleighDampingForce :565-629 with the global matrices.
		vector<double> tmp(n);
		if (alpha != 0.0)
		{
			if (massLumping)  // :584-586: the diagonal of M times v
			{
				for (int c = 0; c < n; ++c)
				{
					double d = 0.0;
					for (int k = pat.colptr[c]; k < pat.colptr[c + 1]; ++k)
						if (pat.rowidx[k] == c) d = M[k];
					tmp[c] = d * V[c];
				}
			}
			else
				spmv(pat, M.data(), V, tmp.data());
			for (int i = 0; i < n; ++i) f[i] -= (1.0 * alpha) * tmp[i];
		}
		if (beta != 0.0)
		{
			spmv(pat, K.data(), V, tmp.data());
			for (int i = 0; i < n; ++i) f[i] -= 1.0 * beta * tmp[i];
		}
		if (hasExternal)  // external generalized force, stiffness, damping (:527-544)
		{
			for (int i = 0; i < n; ++i) f[i] += fExt[i];
			for (int64_t k = 0; k < pat.nnz(); ++k)
			{
				K[k] += kExt[k];
				D[k] += dExt[k];
			}
		}
	}

	// FemRepresentation::update (:232-294) without the compliance matrix.
	int step(double dt)
	{
		if (!active) return ORC_NONFINITE;
		const int n = pat.n;
		xNew.resize(n);
		vNew.resize(n);
		solver.solve(*this, dt, x.data(), v.data(), xNew.data(), vNew.data());
		x.swap(xNew);
		v.swap(vNew);
		hasExternal = false;  // DeformableRepresentation::afterUpdate (DeformableRepresentation.cpp:242-252)
		// OdeState::isValid (OdeState.cpp:268-278): finite sums of positions and velocities.
		double sx = 0, sv = 0;
		for (int i = 0; i < n; ++i)
		{
			sx += x[i];
			sv += v[i];
		}
		if (!std::isfinite(sx) || !std::isfinite(sv))
		{
			active = false;  // setLocalActive(false), :285-293
			return ORC_NONFINITE;
		}
		return solver.stats.cgConverged ? ORC_OK : ORC_CG_MAXITER;
	}
};

// Math/UnitTests/MockObject.h MassPoint: M = m I, D = c I, K = 0, f = m g - c v (3 dofs).
struct MassPointEq : Equation
{
	double mass = 0.456, visc = 0.0, g[3] = {0.0, -9.81, 0.0};
	MassPointEq()
	{
		pat.n = 3;
		pat.colptr = {0, 1, 2, 3};
		pat.rowidx = {0, 1, 2};
		M.assign(3, 0);
		D.assign(3, 0);
		K.assign(3, 0);
		f.assign(3, 0);
	}
	void updateFMDK(const double*, const double* v) override
	{
		for (int i = 0; i < 3; ++i)
		{
			M[i] = mass;
			D[i] = visc;
			K[i] = 0;
			f[i] = mass * g[i] - visc * v[i];
		}
	}
};

}  // namespace

// =============================================================================================
// C interface for the Python test harness (ctypes) and the CPU baseline.
// =============================================================================================
// ---------------------------------------------------------------------------------------------
// Compliance warping rotations (Fem3DCorotationalTetrahedronRepresentation.cpp:112-140): per node,
// the running slerp average of the rotations of the elements holding it, in element order, with the
// i-th rotation (1-based) weighted in by slerp(current, R_i, 1 - 1/i). Quaternions from matrices by the
// largest diagonal combination; slerp along the shorter arc (linear weights when nearly equal).
void quatFromMatrix(const double R[3][3], double q[4])
{
	const double t = R[0][0] + R[1][1] + R[2][2];
	if (t > 0.0)
	{
		const double s = 2.0 * std::sqrt(1.0 + t);
		q[0] = 0.25 * s;
		q[1] = (R[2][1] - R[1][2]) / s;
		q[2] = (R[0][2] - R[2][0]) / s;
		q[3] = (R[1][0] - R[0][1]) / s;
	}
	else if (R[0][0] > R[1][1] && R[0][0] > R[2][2])
	{
		const double s = 2.0 * std::sqrt(1.0 + R[0][0] - R[1][1] - R[2][2]);
		q[0] = (R[2][1] - R[1][2]) / s;
		q[1] = 0.25 * s;
		q[2] = (R[0][1] + R[1][0]) / s;
		q[3] = (R[0][2] + R[2][0]) / s;
	}
	else if (R[1][1] > R[2][2])
	{
		const double s = 2.0 * std::sqrt(1.0 + R[1][1] - R[0][0] - R[2][2]);
		q[0] = (R[0][2] - R[2][0]) / s;
		q[1] = (R[0][1] + R[1][0]) / s;
		q[2] = 0.25 * s;
		q[3] = (R[1][2] + R[2][1]) / s;
	}
	else
	{
		const double s = 2.0 * std::sqrt(1.0 + R[2][2] - R[0][0] - R[1][1]);
		q[0] = (R[1][0] - R[0][1]) / s;
		q[1] = (R[0][2] + R[2][0]) / s;
		q[2] = (R[1][2] + R[2][1]) / s;
		q[3] = 0.25 * s;
	}
}

void matrixFromQuat(const double q[4], double R[3][3])
{
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	R[0][0] = 1 - 2 * (y * y + z * z);
	R[0][1] = 2 * (x * y - w * z);
	R[0][2] = 2 * (x * z + w * y);
	R[1][0] = 2 * (x * y + w * z);
	R[1][1] = 1 - 2 * (x * x + z * z);
	R[1][2] = 2 * (y * z - w * x);
	R[2][0] = 2 * (x * z - w * y);
	R[2][1] = 2 * (y * z + w * x);
	R[2][2] = 1 - 2 * (x * x + y * y);
}

void quatSlerp(const double a[4], const double b[4], double t, double out[4])
{
	const double d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
	const double ad = std::fabs(d);
	double s0, s1;
	if (ad >= 1.0 - DBL_EPSILON)
	{
		s0 = 1.0 - t;
		s1 = t;
	}
	else
	{
		const double th = std::acos(ad), st = std::sin(th);
		s0 = std::sin((1.0 - t) * th) / st;
		s1 = std::sin(t * th) / st;
	}
	if (d < 0.0) s1 = -s1;
	for (int k = 0; k < 4; ++k) out[k] = s0 * a[k] + s1 * b[k];
}

extern "C" {

struct orc_params
{
	double rayleigh_mass;
	double rayleigh_stiffness;
	double gravity[3];
	int32_t gravity_enabled;
	int32_t newton_max_iterations;
	double newton_epsilon;
	double cg_tolerance;
	int32_t cg_max_iterations;  // <= 0: Eigen default 2n
	int32_t element_type;       // 0: corotational tetrahedron, 1: linear tetrahedron, 2: hexahedron
	int32_t mass_lumping;       // FemRepresentation::setMassLumping
};

struct orc_stats
{
	int32_t cg_iterations;
	int32_t newton_iterations;
	int32_t cg_converged;
	int32_t active;
	double cg_error;
	double t_element, t_system, t_solve;
	int32_t singular_g, invalid_rotation, orientation_warnings;
};

void* orc_create(int32_t numNodes, const double* x, int32_t numTets, const int32_t* tets, const double* E,
				 const double* nu, const double* rho, int32_t numBc, const int32_t* bcDofs, const orc_params* prm,
				 int32_t* status)
{
	auto m = std::make_unique<FemModel>();
	*status = ORC_OK;
	if (numNodes <= 0 || numTets <= 0 || !x || !tets || !E || !nu || !rho || !prm)
	{
		*status = ORC_INVALID_ARG;
		return nullptr;
	}
	if (prm->element_type < 0 || prm->element_type > 2)
	{
		*status = ORC_INVALID_ARG;
		return nullptr;
	}
	m->numNodes = numNodes;
	m->xrest.assign(x, x + 3 * (size_t)numNodes);
	m->hex = prm->element_type == 2;
	if (m->hex)
	{
		m->hexes.resize(numTets);
		for (int e = 0; e < numTets; ++e)
		{
			for (int a = 0; a < 8; ++a) m->hexes[e].n[a] = tets[8 * (size_t)e + a];
			m->hexes[e].E = E[e];
			m->hexes[e].nu = nu[e];
			m->hexes[e].rho = rho[e];
		}
	}
	else
	{
		m->tets.resize(numTets);
		for (int e = 0; e < numTets; ++e)
		{
			for (int a = 0; a < 4; ++a) m->tets[e].n[a] = tets[4 * e + a];
			m->tets[e].E = E[e];
			m->tets[e].nu = nu[e];
			m->tets[e].rho = rho[e];
			m->tets[e].linear = prm->element_type == 1;
		}
	}
	std::vector<char> seen(3 * (size_t)numNodes, 0);
	for (int i = 0; i < numBc; ++i)
	{
		int d = bcDofs[i];
		if (d < 0 || d >= 3 * numNodes)
		{
			*status = ORC_INVALID_ARG;
			return nullptr;
		}
		if (!seen[d])  // OdeState::addBoundaryCondition ignores duplicates (OdeState.cpp:134-142)
		{
			seen[d] = 1;
			m->bcDofs.push_back(d);
		}
	}
	m->alpha = prm->rayleigh_mass;
	m->beta = prm->rayleigh_stiffness;
	m->massLumping = prm->mass_lumping != 0;
	for (int k = 0; k < 3; ++k) m->gravity[k] = prm->gravity[k];
	m->gravityEnabled = prm->gravity_enabled != 0;
	m->solver.prm.newtonMaxIter = std::max(1, (int)prm->newton_max_iterations);
	m->solver.prm.newtonEps = prm->newton_epsilon;
	m->solver.prm.cgTol = prm->cg_tolerance;
	m->solver.prm.cgMaxIter = prm->cg_max_iterations > 0 ? prm->cg_max_iterations : -1;
	int st = m->initialize();
	if (st != ORC_OK)
	{
		*status = st;
		return nullptr;
	}
	return m.release();
}

void orc_destroy(void* h) { delete static_cast<FemModel*>(h); }

int64_t orc_nnz(void* h) { return static_cast<FemModel*>(h)->pat.nnz(); }

int32_t orc_step(void* h, double dt, int32_t nsteps, orc_stats* stats)
{
	auto* m = static_cast<FemModel*>(h);
	int st = ORC_OK;
	orc_stats acc{};
	for (int s = 0; s < nsteps; ++s)
	{
		st = m->step(dt);
		acc.cg_iterations += m->solver.stats.cgIterations;
		acc.newton_iterations = m->solver.stats.newtonIterations;
		acc.cg_error = m->solver.stats.cgError;
		acc.t_element += m->solver.stats.tElement;
		acc.t_system += m->solver.stats.tSystem;
		acc.t_solve += m->solver.stats.tSolve;
		if (st == ORC_NONFINITE) break;
	}
	if (stats)
	{
		acc.cg_converged = m->solver.stats.cgConverged;
		acc.active = m->active;
		acc.singular_g = m->singularGCount;
		acc.invalid_rotation = m->invalidRotationCount;
		acc.orientation_warnings = m->orientationWarnings;
		*stats = acc;
	}
	return st;
}

// Seconds of the model's last step by part: element updates and assembly of f, M, D, K; the system
// S, its boundary conditions and the right-hand side; the CG solve.
void orc_last_step_times(void* h, double* t3)
{
	const auto& st = static_cast<FemModel*>(h)->solver.stats;
	t3[0] = st.tElement;
	t3[1] = st.tSystem;
	t3[2] = st.tSolve;
}

void orc_get_state(void* h, double* x, double* v)
{
	auto* m = static_cast<FemModel*>(h);
	if (x) std::copy(m->x.begin(), m->x.end(), x);
	if (v) std::copy(m->v.begin(), m->v.end(), v);
}

void orc_set_state(void* h, const double* x, const double* v)
{
	auto* m = static_cast<FemModel*>(h);
	if (x) std::copy(x, x + m->x.size(), m->x.begin());
	if (v) std::copy(v, v + m->v.size(), m->v.begin());
}

void orc_get_pattern(void* h, int32_t* colptr, int32_t* rowidx)
{
	auto* m = static_cast<FemModel*>(h);
	std::copy(m->pat.colptr.begin(), m->pat.colptr.end(), colptr);
	std::copy(m->pat.rowidx.begin(), m->pat.rowidx.end(), rowidx);
}

void orc_get_scatter(void* h, int32_t* map)
{
	auto* m = static_cast<FemModel*>(h);
	std::copy(m->scatter.begin(), m->scatter.end(), map);
}

// The last assembled system (BC applied) and the F/M/D/K it came from, all in CSC order.
void orc_get_system(void* h, double* S, double* rhs, double* f, double* M, double* D, double* K)
{
	auto* m = static_cast<FemModel*>(h);
	if (S) std::copy(m->solver.S.begin(), m->solver.S.end(), S);
	if (rhs) std::copy(m->solver.rhs.begin(), m->solver.rhs.end(), rhs);
	if (f) std::copy(m->f.begin(), m->f.end(), f);
	if (M) std::copy(m->M.begin(), m->M.end(), M);
	if (D) std::copy(m->D.begin(), m->D.end(), D);
	if (K) std::copy(m->K.begin(), m->K.end(), K);
}

void orc_get_mass_per_node(void* h, double* out)
{
	auto* m = static_cast<FemModel*>(h);
	std::copy(m->massPerNode.begin(), m->massPerNode.end(), out);
}

// Per-element rotation, tangent stiffness, mass and force after the last update.
void orc_get_element(void* h, int32_t e, double* R9, double* K144, double* M144, double* f12)
{
	auto* m = static_cast<FemModel*>(h);
	if (e < 0 || (size_t)e >= m->tets.size()) return;  // tetrahedra only
	const Tet& t = m->tets[e];
	if (R9) std::memcpy(R9, t.R, sizeof(t.R));
	if (K144) std::memcpy(K144, t.K, sizeof(t.K));
	if (M144) std::memcpy(M144, t.M, sizeof(t.M));
	if (f12) std::memcpy(f12, t.f, sizeof(t.f));
}

// Single-element entry point for the element unit tests: rest positions x0 (12), current x (12).
// Outputs V^-1 (16), K0 (144), M0 (144), volume, R (9), K (144), M (144), f (12).
int32_t orc_tet_compute(const double* x0, const double* x, double E, double nu, double rho, double* Vinv16,
						double* K0, double* M0, double* vol, double* R9, double* K, double* M, double* f,
						int32_t* orientationWarning)
{
	Tet t;
	for (int a = 0; a < 4; ++a) t.n[a] = a;
	t.E = E;
	t.nu = nu;
	t.rho = rho;
	int st = tetInitialize(t, x0);
	if (st != ORC_OK) return st;
	if (Vinv16) std::memcpy(Vinv16, t.Vinv, sizeof(t.Vinv));
	if (K0) std::memcpy(K0, t.K0, sizeof(t.K0));
	if (M0) std::memcpy(M0, t.M0, sizeof(t.M0));
	if (vol) *vol = tetVolume(x0, x0 + 3, x0 + 6, x0 + 9);
	if (orientationWarning) *orientationWarning = t.orientationWarning;
	tetUpdateFMDK(t, x);
	if (R9) std::memcpy(R9, t.R, sizeof(t.R));
	if (K) std::memcpy(K, t.K, sizeof(t.K));
	if (M) std::memcpy(M, t.M, sizeof(t.M));
	if (f) std::memcpy(f, t.f, sizeof(t.f));
	return ORC_OK;
}

// Fem3DRepresentation::addExternalGeneralizedForce for the next step (see FemModel::addExternalForce).
int32_t orc_add_external_force(void* h, int32_t element, const double* coord, const double* force,
							   const double* stiffness, const double* damping)
{
	return static_cast<FemModel*>(h)->addExternalForce(element, coord, force, stiffness, damping);
}

// Single hexahedron for the element unit tests: rest positions x0 (24), current x (24). Outputs the
// rest volume, K (576), M (576) and f = -K (x - x0) (24); ORC_DEGENERATE as Fem3DElementCube asserts.
int32_t orc_hex_compute(const double* x0, const double* x, double E, double nu, double rho, double* vol, double* K,
						double* M, double* f)
{
	Hex t;
	for (int a = 0; a < 8; ++a) t.n[a] = a;
	t.E = E;
	t.nu = nu;
	t.rho = rho;
	int st = hexInitialize(t, x0);
	if (st != ORC_OK) return st;
	if (vol) *vol = t.volume;
	if (K) std::memcpy(K, t.K0, sizeof(t.K0));
	if (M) std::memcpy(M, t.M0, sizeof(t.M0));
	if (x && f)
	{
		hexUpdateF(t, x);
		std::memcpy(f, t.f, sizeof(t.f));
	}
	return ORC_OK;
}

// Shape function i and its three natural derivatives at (eps, eta, mu).
void orc_hex_shape(int32_t i, double e, double h, double m, double* out4)
{
	out4[0] = hexN(i, e, h, m);
	out4[1] = hexdNde(i, e, h, m);
	out4[2] = hexdNdh(i, e, h, m);
	out4[3] = hexdNdm(i, e, h, m);
}

void orc_polar(const double* F9, double* R9, double* S9)
{
	double F[3][3], R[3][3], S[3][3];
	std::memcpy(F, F9, sizeof(F));
	polar33(F, R, S);
	std::memcpy(R9, R, sizeof(R));
	std::memcpy(S9, S, sizeof(S));
}

// LinearSparseSolveAndInverseCG::solve on a caller CSC matrix.
// DeformableRepresentation::applyCompliance (DeformableRepresentation.cpp:175-191): for each column of
// b (column-major n x ncols), zero the BC rows, solve with the last step's system matrix, zero the BC
// rows of the solution; with warping, FemRepresentation::applyCompliance (FemRepresentation.cpp:329-340):
// W (that applied to W^T b), W the per-node rotations of the last element update. Returns ORC_CG_MAXITER
// if a column's solve did not converge.
int32_t orc_apply_compliance(void* h, int32_t ncols, const double* b, double* x, int32_t warping, int32_t* iterations)
{
	auto* m = static_cast<FemModel*>(h);
	const int n = m->pat.n, N = n / 3;
	if (ncols < 0 || (ncols > 0 && (!b || !x)) || m->solver.S.empty()) return ORC_INVALID_ARG;
	if (warping && m->hex) return ORC_INVALID_ARG;  // warping rotations are the corotational tetrahedra's
	vector<double> W;
	if (warping)
	{
		W.assign(9 * (size_t)N, 0.0);
		vector<vector<int>> inc(N);
		for (size_t e = 0; e < m->tets.size(); ++e)
			for (int a = 0; a < 4; ++a) inc[m->tets[e].n[a]].push_back((int)e);
		for (int I = 0; I < N; ++I)
		{
			double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
			if (!inc[I].empty())
			{
				double q[4];
				quatFromMatrix(m->tets[inc[I][0]].R, q);
				for (size_t i = 2; i <= inc[I].size(); ++i)
				{
					double qe[4], qn[4];
					quatFromMatrix(m->tets[inc[I][i - 1]].R, qe);
					quatSlerp(q, qe, 1.0 - 1.0 / (double)i, qn);
					std::copy(qn, qn + 4, q);
				}
				matrixFromQuat(q, R);
			}
			for (int i = 0; i < 3; ++i)
				for (int j = 0; j < 3; ++j) W[9 * (size_t)I + 3 * i + j] = R[i][j];
		}
	}
	int32_t st = ORC_OK;
	int32_t its = 0;
	vector<double> col(n), sol(n);
	for (int c = 0; c < ncols; ++c)
	{
		const double* bc = b + (size_t)c * n;
		for (int I = 0; I < N; ++I)
			for (int i = 0; i < 3; ++i)
			{
				if (!warping)
					col[3 * I + i] = bc[3 * I + i];
				else
				{
					const double* w = &W[9 * (size_t)I];
					col[3 * I + i] = w[i] * bc[3 * I] + w[3 + i] * bc[3 * I + 1] + w[6 + i] * bc[3 * I + 2];
				}
			}
		for (int d : m->bcDofs) col[d] = 0.0;
		CgResult cr = cgSolve(m->pat, m->solver.S.data(), col.data(), sol.data(), m->solver.prm.cgTol,
							  m->solver.prm.cgMaxIter);
		its += cr.iterations;
		if (!cr.converged) st = ORC_CG_MAXITER;
		for (int d : m->bcDofs) sol[d] = 0.0;
		double* xc = x + (size_t)c * n;
		for (int I = 0; I < N; ++I)
			for (int i = 0; i < 3; ++i)
			{
				if (!warping)
					xc[3 * I + i] = sol[3 * I + i];
				else
				{
					const double* w = &W[9 * (size_t)I + 3 * i];
					xc[3 * I + i] = w[0] * sol[3 * I] + w[1] * sol[3 * I + 1] + w[2] * sol[3 * I + 2];
				}
			}
	}
	if (iterations) *iterations = its;
	return st;
}

int32_t orc_cg_solve(int32_t n, const int32_t* colptr, const int32_t* rowidx, const double* vals, const double* b,
					 double* x, double tol, int32_t maxIter, int32_t* iterations, double* error)
{
	Pattern p;
	p.n = n;
	p.colptr.assign(colptr, colptr + n + 1);
	p.rowidx.assign(rowidx, rowidx + colptr[n]);
	CgResult r = cgSolve(p, vals, b, x, tol, maxIter > 0 ? maxIter : -1);
	if (iterations) *iterations = r.iterations;
	if (error) *error = r.error;
	return r.converged ? ORC_OK : ORC_CG_MAXITER;
}

// OdeSolverEulerImplicit on the MassPoint mock (OdeSolverEulerImplicitTests.cpp:58-115).
void orc_masspoint_step(double viscosity, double dt, const double* x0, const double* v0, double* x1, double* v1)
{
	MassPointEq eq;
	eq.visc = viscosity;
	ImplicitEuler s;
	s.prm.cgTol = 1e-14;
	s.solve(eq, dt, x0, v0, x1, v1);
}

// Independent models stepped by a worker pool of `threads` threads: every step enqueues one task
// per model and waits for all of them (FreeMotion.cpp:55-80; the pool size of Runtime.cpp:349-359
// is chosen by the caller).
int32_t orc_step_many(void** models, int32_t count, double dt, int32_t nsteps, int32_t threads)
{
	int worstAll = 0;
	for (int s = 0; s < nsteps; ++s)
	{
		std::atomic<int> next{0};
		std::atomic<int> worst{0};
		auto worker = [&]() {
			for (;;)
			{
				int i = next.fetch_add(1);
				if (i >= count) break;
				int st = orc_step(models[i], dt, 1, nullptr);
				int w = worst.load();
				while (st > w && !worst.compare_exchange_weak(w, st)) {}
			}
		};
		std::vector<std::thread> pool;
		for (int t = 0; t < std::max(1, (int)threads); ++t) pool.emplace_back(worker);
		for (auto& t : pool) t.join();
		worstAll = std::max(worstAll, worst.load());
	}
	return worstAll;
}

}  // extern "C"
