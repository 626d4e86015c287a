// Test support only: a C++ program written against the OpenSurgSim-named facade
// (include/surgsim_compat/surgsim_gb300.h), as a reference-side caller would use it.
//
//   facade_c1 <mesh.bin> <out.bin> <steps>
//
// mesh.bin: int32 N, int32 E, int32 B, double[3N] vertices, int32[4E] tetrahedra, double[E] E,
// double[E] nu, double[E] rho, int32[B] boundary-condition vertices, double alpha, double beta,
// double[3] gravity, double dt, double cg tolerance.
// It builds a Fem3DRepresentation with corotational tetrahedra, EULER_IMPLICIT and CONJUGATEGRADIENT,
// checks that the unsupported schemes and solvers throw, runs `steps` updates, then one
// OdeSolverEulerImplicit::solve from the current state with its system matrix and (small bodies)
// the compliance matrix, and one applyCompliance. out.bin: x, v after the updates (3N each); x, v
// of the solve's new state; nnz and the system matrix values (CSC); the compliance matrix (n x n,
// column-major, or nothing when n > 600); applyCompliance of two columns (n x 2).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "surgsim_compat/surgsim_gb300.h"

using namespace surgsim_gb300;

template <typename T>
static void rd(FILE* f, T* p, size_t n)
{
	if (fread(p, sizeof(T), n, f) != n)
	{
		fprintf(stderr, "short read\n");
		exit(3);
	}
}

template <typename T>
static void wr(FILE* f, const T* p, size_t n)
{
	fwrite(p, sizeof(T), n, f);
}

int main(int argc, char** argv)
{
	if (argc != 4) return 2;
	FILE* in = fopen(argv[1], "rb");
	if (!in) return 2;
	int32_t N, E, B;
	rd(in, &N, 1);
	rd(in, &E, 1);
	rd(in, &B, 1);
	Physics::Fem3D mesh;
	mesh.vertices.resize(3 * (size_t)N);
	mesh.tetrahedra.resize(4 * (size_t)E);
	mesh.youngModulus.resize(E);
	mesh.poissonRatio.resize(E);
	mesh.massDensity.resize(E);
	mesh.boundaryConditions.resize(B);
	rd(in, mesh.vertices.data(), mesh.vertices.size());
	rd(in, mesh.tetrahedra.data(), mesh.tetrahedra.size());
	rd(in, mesh.youngModulus.data(), E);
	rd(in, mesh.poissonRatio.data(), E);
	rd(in, mesh.massDensity.data(), E);
	rd(in, mesh.boundaryConditions.data(), B);
	double alpha, beta, g[3], dt, tol;
	rd(in, &alpha, 1);
	rd(in, &beta, 1);
	rd(in, g, 3);
	rd(in, &dt, 1);
	rd(in, &tol, 1);
	fclose(in);
	const int steps = atoi(argv[3]);

	Physics::Fem3DRepresentation fem("c1");
	fem.setFem(mesh);
	fem.setFemElementType("SurgSim::Physics::Fem3DElementCorotationalTetrahedron");
	// Schemes and solvers this path does not provide are refused, not ignored.
	int refused = 0;
	for (Math::IntegrationScheme s : {Math::INTEGRATIONSCHEME_EULER_EXPLICIT, Math::INTEGRATIONSCHEME_STATIC,
									  Math::INTEGRATIONSCHEME_RUNGE_KUTTA_4, Math::INTEGRATIONSCHEME_LINEAR_EULER_IMPLICIT})
	{
		try
		{
			fem.setIntegrationScheme(s);
		}
		catch (const Framework::AssertionFailure&)
		{
			++refused;
		}
	}
	try
	{
		fem.setLinearSolver(Math::LINEARSOLVER_LU);
	}
	catch (const Framework::AssertionFailure&)
	{
		++refused;
	}
	if (refused != 5) return 4;
	fem.setIntegrationScheme(Math::INTEGRATIONSCHEME_EULER_IMPLICIT);
	fem.setLinearSolver(Math::LINEARSOLVER_CONJUGATEGRADIENT);
	fem.setRayleighDampingMass(alpha);
	fem.setRayleighDampingStiffness(beta);
	fem.setGravity(g[0], g[1], g[2]);
	fem.setLinearSolverTolerance(tol);
	fem.initialize();
	try
	{
		fem.setMassLumping(true);  // FemRepresentation: not after initialization
		return 5;
	}
	catch (const Framework::AssertionFailure&)
	{
	}
	auto solver = fem.getOdeSolver();
	if (!solver || solver->getName() != "Ode Solver Euler Implicit") return 6;
	for (int s = 0; s < steps; ++s) fem.update(dt);
	if (!fem.isActive()) return 7;
	const Math::OdeState cur = fem.getCurrentState();

	FILE* out = fopen(argv[2], "wb");
	if (!out) return 2;
	wr(out, cur.positions.data(), cur.positions.size());
	wr(out, cur.velocities.data(), cur.velocities.size());

	// OdeSolverEulerImplicit::solve from the current state; the representation's state is unchanged.
	Math::OdeState next;
	const int32_t n = (int32_t)cur.getNumDof();
	const bool small = n <= 600;
	solver->solve(dt, cur, &next, small);
	const Math::OdeState after = fem.getCurrentState();
	if (after.positions != cur.positions || after.velocities != cur.velocities) return 8;
	wr(out, next.positions.data(), next.positions.size());
	wr(out, next.velocities.data(), next.velocities.size());
	const Math::SparseMatrix& S = solver->getSystemMatrix();
	const int64_t nnz = S.nonZeros();
	wr(out, &nnz, 1);
	wr(out, S.values.data(), S.values.size());
	if (small)
	{
		const Math::Matrix& C = solver->getComplianceMatrix();
		if (C.rows != n || C.cols != n) return 9;
		wr(out, C.data.data(), C.data.size());
	}
	Math::Matrix b(n, 2);
	for (int32_t i = 0; i < n; ++i)
	{
		b(i, 0) = 1.0 + 0.001 * i;
		b(i, 1) = (i % 3 == 2) ? -1.0 : 0.5;
	}
	const Math::Matrix x = fem.applyCompliance(cur, b);
	wr(out, x.data.data(), x.data.size());
	fclose(out);
	return 0;
}
