// surgsim_gb300.h -- header-only C++ facade over the gbfem C ABI that keeps OpenSurgSim's class and
// method names for the FEM-3D implicit-Euler path, so code written against
//   SurgSim::Physics::Fem3DRepresentation   (Physics/Fem3DRepresentation.h, FemRepresentation.h,
//                                            DeformableRepresentation.h)
//   SurgSim::Math::OdeSolverEulerImplicit   (Math/OdeSolverEulerImplicit.h, Math/OdeSolver.h:78-159)
//   SurgSim::Math::LinearSparseSolveAndInverseCG (Math/LinearSparseSolveAndInverse.h:98-123)
// can switch to the GB300 step by changing the namespace. Failures throw AssertionFailure (the
// reference's SurgSim::Framework::AssertionFailure, Framework/Assert.h:77-95) carrying the
// message of gbfem_last_error; a representation whose state stops being finite is deactivated
// instead, as in FemRepresentation::update (FemRepresentation.cpp:285-293).
//
// What the path supports, and what throws: the integration schemes EULER_IMPLICIT (any element
// type) and LINEAR_EULER_IMPLICIT (linear elements: Fem3DElementTetrahedron, Fem3DElementCube); the
// linear solver CONJUGATEGRADIENT. Every other scheme or solver of the reference throws
// AssertionFailure from its setter, instead of being accepted and ignored.
#pragma once

#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "../gbfem.h"

namespace surgsim_gb300 {

namespace Framework {
class AssertionFailure : public std::runtime_error
{
public:
	explicit AssertionFailure(const std::string& msg) : std::runtime_error(msg) {}
};
}  // namespace Framework

namespace detail {
inline std::string lastError(gbfem_handle h)
{
	char buf[1024];
	gbfem_last_error(h, buf, sizeof(buf));
	return buf;
}
inline void check(gbfem_status st, gbfem_handle h, const char* what)
{
	if (st != GBFEM_OK) throw Framework::AssertionFailure(std::string(what) + ": " + lastError(h));
}
}  // namespace detail

namespace Math {

// The reference's IntegrationScheme and LinearSolver enums with their values (Math/OdeSolver.h:36-48,
// Math/LinearSparseSolveAndInverse.h:41-46).
enum IntegrationScheme
{
	INTEGRATIONSCHEME_STATIC = 0,
	INTEGRATIONSCHEME_LINEAR_STATIC,
	INTEGRATIONSCHEME_EULER_EXPLICIT,
	INTEGRATIONSCHEME_LINEAR_EULER_EXPLICIT,
	INTEGRATIONSCHEME_EULER_EXPLICIT_MODIFIED,
	INTEGRATIONSCHEME_LINEAR_EULER_EXPLICIT_MODIFIED,
	INTEGRATIONSCHEME_EULER_IMPLICIT,
	INTEGRATIONSCHEME_LINEAR_EULER_IMPLICIT,
	INTEGRATIONSCHEME_RUNGE_KUTTA_4,
	INTEGRATIONSCHEME_LINEAR_RUNGE_KUTTA_4,
	INTEGRATIONSCHEME_COUNT
};
enum LinearSolver
{
	LINEARSOLVER_LU = 0,
	LINEARSOLVER_CONJUGATEGRADIENT,
	LINEARSOLVER_COUNT
};

// SurgSim::Math::SparseMatrix is Eigen::SparseMatrix<double, ColMajor, int> (Math/SparseMatrix.h:32):
// compressed columns, rows sorted within a column, explicit zeros kept.
struct SparseMatrix
{
	int32_t rows = 0, cols = 0;
	std::vector<int32_t> colptr, rowidx;
	std::vector<double> values;
	int64_t nonZeros() const { return (int64_t)values.size(); }
	// Entry (r, c), 0 when outside the pattern (Eigen's coeff).
	double coeff(int32_t r, int32_t c) const
	{
		for (int32_t k = colptr[c]; k < colptr[c + 1]; ++k)
			if (rowidx[k] == r) return values[k];
		return 0.0;
	}
};

// SurgSim::Math::Matrix is a dense column-major Eigen::MatrixXd (Math/Matrix.h).
struct Matrix
{
	int32_t rows = 0, cols = 0;
	std::vector<double> data;  // column-major
	Matrix() = default;
	Matrix(int32_t r, int32_t c) : rows(r), cols(c), data((size_t)r * c, 0.0) {}
	static Matrix Identity(int32_t r, int32_t c)
	{
		Matrix m(r, c);
		for (int32_t i = 0; i < r && i < c; ++i) m(i, i) = 1.0;
		return m;
	}
	double& operator()(int32_t r, int32_t c) { return data[(size_t)c * rows + r]; }
	double operator()(int32_t r, int32_t c) const { return data[(size_t)c * rows + r]; }
};

// Positions and velocities of a representation (Math/OdeState.h), node-major x,y,z.
struct OdeState
{
	std::vector<double> positions, velocities;
	const std::vector<double>& getPositions() const { return positions; }
	const std::vector<double>& getVelocities() const { return velocities; }
	std::vector<double>& getPositions() { return positions; }
	std::vector<double>& getVelocities() { return velocities; }
	size_t getNumDof() const { return positions.size(); }
	size_t getNumNodes() const { return positions.size() / 3; }
};

// The equation an OdeSolver solves (Math/OdeEquation.h:54-143). Here it is the GPU body of a
// representation; Physics::Fem3DRepresentation implements it.
class OdeEquation
{
public:
	virtual ~OdeEquation() = default;
	virtual gbfem_handle odeHandle() const = 0;
	// Element type of the body (GBFEM_ELEMENT_*): what the system matrix export supports.
	virtual int32_t odeElementType() const = 0;
	virtual gbfem_precision odePrecision() const = 0;
};

// LinearSparseSolveAndInverseCG on the GPU: setMatrix takes a CSC matrix (Eigen ColMajor), of
// which only the lower triangle is read, as Eigen's ConjugateGradient<..., Lower> does.
class LinearSparseSolveAndInverseCG
{
public:
	void setTolerance(double tolerance)
	{
		m_tolerance = tolerance;
		if (m_cg) gbfem_cg_set_tolerance(m_cg.get(), tolerance);
	}
	double getTolerance() const { return m_tolerance; }
	void setMaxIterations(int32_t iterations)
	{
		m_maxIterations = iterations;
		if (m_cg) gbfem_cg_set_max_iterations(m_cg.get(), iterations);
	}
	int32_t getMaxIterations() const { return m_maxIterations; }
	void setMatrix(int32_t n, const std::vector<int32_t>& colptr, const std::vector<int32_t>& rowidx,
				   const std::vector<double>& values, int32_t device = 0)
	{
		if ((int32_t)colptr.size() != n + 1) throw Framework::AssertionFailure("Cannot inverse a non square matrix");
		gbfem_cg cg = nullptr;
		detail::check(gbfem_cg_create(n, colptr.data(), rowidx.data(), values.data(), device, &cg), nullptr,
					  "LinearSparseSolveAndInverseCG::setMatrix");
		m_cg.reset(cg);
		m_n = n;
		gbfem_cg_set_tolerance(cg, m_tolerance);
		gbfem_cg_set_max_iterations(cg, m_maxIterations);
	}
	void setMatrix(const SparseMatrix& A, int32_t device = 0)
	{
		if (A.rows != A.cols) throw Framework::AssertionFailure("Cannot inverse a non square matrix");
		setMatrix(A.rows, A.colptr, A.rowidx, A.values, device);
	}
	std::vector<double> solve(const std::vector<double>& b) const
	{
		if (!m_cg || (int32_t)b.size() != m_n) throw Framework::AssertionFailure("solve: matrix not set or size mismatch");
		std::vector<double> x(b.size());
		int32_t it = 0;
		double res = 0;
		gbfem_status st = gbfem_cg_solve(m_cg.get(), b.data(), x.data(), &it, &res);
		if (st != GBFEM_OK && st != GBFEM_CG_MAXITER) detail::check(st, nullptr, "LinearSparseSolveAndInverseCG::solve");
		m_lastIterations = it;
		m_lastError = res;
		return x;  // like the reference, reaching maxIterations is not an error
	}
	int32_t lastIterations() const { return m_lastIterations; }
	double lastError() const { return m_lastError; }

private:
	struct Deleter
	{
		void operator()(gbfem_cg_s* c) const { gbfem_cg_destroy(c); }
	};
	std::unique_ptr<gbfem_cg_s, Deleter> m_cg;
	int32_t m_n = 0;
	double m_tolerance = 2.220446049250313e-16;  // Eigen's default: NumTraits<double>::epsilon()
	int32_t m_maxIterations = 0;                 // <= 0: Eigen's default 2n
	mutable int32_t m_lastIterations = 0;
	mutable double m_lastError = 0;
};

// OdeSolverEulerImplicit (Math/OdeSolverEulerImplicit.cpp:25-161) over the equation's GPU body. The
// solver's Newton settings and its linear solver's tolerance and iteration cap are pushed to the
// body before every solve. solve() steps from currentState and leaves the equation's own state as it
// was (the reference's solver writes only newState). The system matrix of the last solve (or
// computeMatrices) is read back from the device; the export needs the FP64 form and tetrahedra
// (GBFEM_STEP_KEEP_SYSTEM), otherwise getSystemMatrix throws. The compliance matrix is the dense
// inverse of that system with the boundary-condition rows and columns zeroed
// (OdeSolver.cpp:69-76), formed column by column by the body's multi-right-hand-side CG
// (gbfem_apply_compliance on the identity): O(n) solves, meant for small bodies, as in the
// reference.
class OdeSolverEulerImplicit
{
public:
	explicit OdeSolverEulerImplicit(OdeEquation* equation) : m_equation(equation)
	{
		if (!equation) throw Framework::AssertionFailure("OdeSolverEulerImplicit needs an equation");
		m_linearSolver = std::make_shared<LinearSparseSolveAndInverseCG>();
	}
	const std::string getName() const { return "Ode Solver Euler Implicit"; }

	void setLinearSolver(std::shared_ptr<LinearSparseSolveAndInverseCG> linearSolver)
	{
		if (!linearSolver) throw Framework::AssertionFailure("setLinearSolver: null linear solver");
		m_linearSolver = linearSolver;
	}
	std::shared_ptr<LinearSparseSolveAndInverseCG> getLinearSolver() const { return m_linearSolver; }

	void setNewtonRaphsonMaximumIteration(size_t maximumIteration)
	{
		if (maximumIteration < 1) throw Framework::AssertionFailure("The maximum iteration needs to be at least 1");
		m_maximumIteration = maximumIteration;
	}
	size_t getNewtonRaphsonMaximumIteration() const { return m_maximumIteration; }
	void setNewtonRaphsonEpsilonConvergence(double epsilonConvergence)
	{
		if (epsilonConvergence < 0) throw Framework::AssertionFailure("The epsilon convergence cannot be negative");
		m_epsilonConvergence = epsilonConvergence;
	}
	double getNewtonRaphsonEpsilonConvergence() const { return m_epsilonConvergence; }

	// OdeSolver::solve (:106): newState = the implicit-Euler step of dt from currentState.
	void solve(double dt, const OdeState& currentState, OdeState* newState, bool computeCompliance = true)
	{
		if (!newState) throw Framework::AssertionFailure("OdeSolverEulerImplicit::solve: newState is null");
		gbfem_handle h = handle();
		const OdeState saved = readState(h);
		if (currentState.positions.size() != saved.positions.size() ||
			currentState.velocities.size() != saved.velocities.size())
			throw Framework::AssertionFailure("OdeSolverEulerImplicit::solve: state size mismatch");
		pushSettings(h);
		detail::check(gbfem_set_state(h, currentState.positions.data(), currentState.velocities.data()), h,
					  "OdeSolverEulerImplicit::solve");
		const gbfem_status st = gbfem_step(h, dt, 1, keepFlag());
		if (st != GBFEM_OK && st != GBFEM_CG_MAXITER && st != GBFEM_NONFINITE)
			detail::check(st, h, "OdeSolverEulerImplicit::solve");
		*newState = readState(h);
		if (st == GBFEM_NONFINITE) gbfem_reactivate(h);  // the representation decides on deactivation
		m_haveSystem = keepFlag() != 0;
		if (computeCompliance) computeComplianceMatrixFromSystemMatrix();
		detail::check(gbfem_set_state(h, saved.positions.data(), saved.velocities.data()), h,
					  "OdeSolverEulerImplicit::solve");
	}

	// OdeSolver::computeMatrices (:112, OdeSolver.cpp:58-67): the system matrix at `state`
	// (assembleLinearSystem with state as both states) and, if asked, the compliance matrix.
	void computeMatrices(double dt, const OdeState& state, bool computeCompliance = true)
	{
		OdeState unused;
		const size_t iters = m_maximumIteration;
		m_maximumIteration = 1;  // one assembly at `state`, as assembleLinearSystem(dt, state, state)
		try
		{
			solve(dt, state, &unused, computeCompliance);
		}
		catch (...)
		{
			m_maximumIteration = iters;
			throw;
		}
		m_maximumIteration = iters;
	}

	// OdeSolver::getSystemMatrix (:116): S = M/dt + D + dt K of the last solve with the boundary
	// conditions applied (rows and columns zeroed, 1 on the diagonal), full (both triangles).
	const SparseMatrix& getSystemMatrix() const
	{
		if (!m_haveSystem)
			throw Framework::AssertionFailure(
				"getSystemMatrix: no system matrix (solve first; the export needs the FP64 form and tetrahedra)");
		gbfem_handle h = handle();
		int64_t n = 0, nnz = 0;
		detail::check(gbfem_get_sizes(h, &n, &nnz), h, "getSystemMatrix");
		m_system.rows = m_system.cols = (int32_t)n;
		m_system.colptr.resize(n + 1);
		m_system.rowidx.resize(nnz);
		m_system.values.resize(nnz);
		detail::check(gbfem_get_pattern(h, m_system.colptr.data(), m_system.rowidx.data()), h, "getSystemMatrix");
		std::vector<double> rhs(n), f(n);
		detail::check(gbfem_get_system(h, m_system.values.data(), rhs.data(), f.data()), h, "getSystemMatrix");
		return m_system;
	}
	// OdeSolver::getComplianceMatrix (:119).
	const Matrix& getComplianceMatrix() const { return m_compliance; }

private:
	gbfem_handle handle() const
	{
		gbfem_handle h = m_equation->odeHandle();
		if (!h) throw Framework::AssertionFailure("OdeSolverEulerImplicit: the equation is not initialized");
		return h;
	}
	uint32_t keepFlag() const
	{
		const bool tets = m_equation->odeElementType() != GBFEM_ELEMENT_HEXAHEDRON;
		return (tets && m_equation->odePrecision() == GBFEM_PRECISION_FP64) ? GBFEM_STEP_KEEP_SYSTEM : 0u;
	}
	void pushSettings(gbfem_handle h) const
	{
		detail::check(gbfem_set_solver_params(h, (int32_t)m_maximumIteration, m_epsilonConvergence,
											  m_linearSolver->getTolerance(), m_linearSolver->getMaxIterations()),
					  h, "OdeSolverEulerImplicit");
	}
	static OdeState readState(gbfem_handle h)
	{
		OdeState s;
		int64_t n = 0, nnz = 0;
		gbfem_get_sizes(h, &n, &nnz);
		s.positions.resize(n);
		s.velocities.resize(n);
		detail::check(gbfem_get_state(h, s.positions.data(), s.velocities.data()), h, "OdeState");
		return s;
	}
	void computeComplianceMatrixFromSystemMatrix()
	{
		gbfem_handle h = handle();
		int64_t n = 0, nnz = 0;
		gbfem_get_sizes(h, &n, &nnz);
		const Matrix I = Matrix::Identity((int32_t)n, (int32_t)n);
		m_compliance = Matrix((int32_t)n, (int32_t)n);
		const gbfem_status st = gbfem_apply_compliance(h, (int32_t)n, I.data.data(), m_compliance.data.data(), 0, nullptr);
		if (st != GBFEM_CG_MAXITER) detail::check(st, h, "computeComplianceMatrixFromSystemMatrix");
	}

	OdeEquation* m_equation;  // non-owning, as OdeSolver::m_equation (OdeSolver.cpp:25)
	std::shared_ptr<LinearSparseSolveAndInverseCG> m_linearSolver;
	size_t m_maximumIteration = 1;       // OdeSolverEulerImplicit.cpp:25-29
	double m_epsilonConvergence = 1e-5;
	bool m_haveSystem = false;
	mutable SparseMatrix m_system;
	Matrix m_compliance;
};

}  // namespace Math

namespace Physics {

// Volume mesh in the form Fem3D carries it (vertices, 4- or 8-node elements with their material,
// boundary-condition vertices), cf. Physics/Fem3DRepresentation.cpp:70-126.
struct Fem3D
{
	std::vector<double> vertices;          // 3 * N
	std::vector<int32_t> tetrahedra;       // 4 * E (tetrahedral element types)
	std::vector<int32_t> cubes;            // 8 * E (SurgSim::Physics::Fem3DElementCube)
	std::vector<double> youngModulus, poissonRatio, massDensity;  // E each
	std::vector<int32_t> boundaryConditions;  // vertex ids; all 3 dofs of each are fixed
};

class Fem3DRepresentation : public Math::OdeEquation
{
public:
	explicit Fem3DRepresentation(const std::string& name) : m_name(name) { gbfem_params_default(&m_params); }

	const std::string& getName() const { return m_name; }
	void setFem(const Fem3D& mesh)
	{
		if (m_handle) throw Framework::AssertionFailure("The Fem cannot be set after initialization");
		m_mesh = mesh;
	}
	// The element factory names of the three provided element types.
	void setFemElementType(const std::string& type)
	{
		if (m_handle) throw Framework::AssertionFailure("The element type cannot be set after initialization");
		if (type == "SurgSim::Physics::Fem3DElementCorotationalTetrahedron")
			m_params.element_type = GBFEM_ELEMENT_COROTATIONAL_TET;
		else if (type == "SurgSim::Physics::Fem3DElementTetrahedron")
			m_params.element_type = GBFEM_ELEMENT_LINEAR_TET;
		else if (type == "SurgSim::Physics::Fem3DElementCube")
			m_params.element_type = GBFEM_ELEMENT_HEXAHEDRON;
		else
			throw Framework::AssertionFailure("unsupported element type " + type);
		m_elementType = type;
		checkScheme(m_scheme);
	}
	const std::string& getFemElementType() const { return m_elementType; }
	// DeformableRepresentation::setIntegrationScheme (DeformableRepresentation.h:92): EULER_IMPLICIT,
	// or LINEAR_EULER_IMPLICIT with a linear element type; any other scheme throws.
	void setIntegrationScheme(Math::IntegrationScheme scheme)
	{
		if (m_handle) throw Framework::AssertionFailure("The integration scheme cannot be set after initialization");
		checkScheme(scheme);
		m_scheme = scheme;
	}
	Math::IntegrationScheme getIntegrationScheme() const { return m_scheme; }
	// DeformableRepresentation::setLinearSolver (DeformableRepresentation.h:106): CONJUGATEGRADIENT only.
	void setLinearSolver(Math::LinearSolver solver)
	{
		if (solver != Math::LINEARSOLVER_CONJUGATEGRADIENT)
			throw Framework::AssertionFailure("unsupported linear solver: this path solves with LINEARSOLVER_CONJUGATEGRADIENT");
		m_linearSolver = solver;
	}
	Math::LinearSolver getLinearSolver() const { return m_linearSolver; }
	void setRayleighDampingMass(double c) { m_params.rayleigh_mass = c; }
	void setRayleighDampingStiffness(double c) { m_params.rayleigh_stiffness = c; }
	// FemRepresentation::setMassLumping (FemRepresentation.cpp:320-323): before initialization only.
	void setMassLumping(bool useMassLumping)
	{
		if (m_handle) throw Framework::AssertionFailure("Can't change mass lumping after initialization.");
		m_params.mass_lumping = useMassLumping ? 1 : 0;
	}
	bool getMassLumping() const { return m_params.mass_lumping != 0; }
	// FemRepresentation::setComplianceWarping: applyCompliance with W S^-1 W^T (corotational elements).
	void setComplianceWarping(bool on)
	{
		if (m_handle) throw Framework::AssertionFailure("Compliance warping cannot be modified once the component is initialized");
		m_complianceWarping = on;
	}
	bool getComplianceWarping() const { return m_complianceWarping; }
	void setIsGravityEnabled(bool on) { m_params.gravity_enabled = on ? 1 : 0; }
	// The reference's gravity is fixed at (0, -9.81, 0) (Representation.cpp:36); this one can be set.
	void setGravity(double gx, double gy, double gz)
	{
		m_params.gravity[0] = gx;
		m_params.gravity[1] = gy;
		m_params.gravity[2] = gz;
	}
	// OdeSolverEulerImplicit settings (OdeSolverEulerImplicit.cpp:31-53), forwarded to the solver
	// once it exists.
	void setNewtonRaphsonMaximumIteration(int32_t n)
	{
		if (n < 1) throw Framework::AssertionFailure("The maximum iteration needs to be at least 1");
		m_params.newton_max_iterations = n;
		if (m_odeSolver) m_odeSolver->setNewtonRaphsonMaximumIteration((size_t)n);
	}
	void setNewtonRaphsonEpsilonConvergence(double eps)
	{
		if (eps < 0) throw Framework::AssertionFailure("The epsilon convergence cannot be negative");
		m_params.newton_epsilon = eps;
		if (m_odeSolver) m_odeSolver->setNewtonRaphsonEpsilonConvergence(eps);
	}
	// LinearSparseSolveAndInverseCG settings.
	void setLinearSolverTolerance(double tol)
	{
		m_params.cg_tolerance = tol;
		if (m_odeSolver) m_odeSolver->getLinearSolver()->setTolerance(tol);
	}
	void setLinearSolverMaxIterations(int32_t it)
	{
		m_params.cg_max_iterations = it;
		if (m_odeSolver) m_odeSolver->getLinearSolver()->setMaxIterations(it);
	}
	// GB300 extension: FP64 plain form or FP32 with FP64 refinement.
	void setPrecision(gbfem_precision p)
	{
		if (m_handle) throw Framework::AssertionFailure("The precision cannot be set after initialization");
		m_params.precision = p;
	}
	void setDevice(int32_t device) { m_params.device = device; }

	// Representation::initialize + wakeUp: builds the device body and its OdeSolverEulerImplicit
	// (DeformableRepresentation::doInitialize, DeformableRepresentation.cpp:334-385).
	bool initialize()
	{
		gbfem_mesh_desc d{};
		d.num_nodes = (int32_t)(m_mesh.vertices.size() / 3);
		d.rest_positions = m_mesh.vertices.data();
		const bool cube = m_params.element_type == GBFEM_ELEMENT_HEXAHEDRON;
		d.num_tets = cube ? (int32_t)(m_mesh.cubes.size() / 8) : (int32_t)(m_mesh.tetrahedra.size() / 4);
		d.tets = cube ? m_mesh.cubes.data() : m_mesh.tetrahedra.data();
		d.young_modulus = m_mesh.youngModulus.data();
		d.poisson_ratio = m_mesh.poissonRatio.data();
		d.mass_density = m_mesh.massDensity.data();
		std::vector<int32_t> dofs;
		for (int32_t node : m_mesh.boundaryConditions)
			for (int k = 0; k < 3; ++k) dofs.push_back(3 * node + k);
		d.num_bc_dofs = (int32_t)dofs.size();
		d.bc_dofs = dofs.data();
		gbfem_handle h = nullptr;
		detail::check(gbfem_create(&d, &m_params, &h), nullptr, "Fem3DRepresentation::initialize");
		m_handle.reset(h);
		m_odeSolver = std::make_shared<Math::OdeSolverEulerImplicit>(this);
		m_odeSolver->setNewtonRaphsonMaximumIteration((size_t)m_params.newton_max_iterations);
		m_odeSolver->setNewtonRaphsonEpsilonConvergence(m_params.newton_epsilon);
		m_odeSolver->getLinearSolver()->setTolerance(m_params.cg_tolerance);
		m_odeSolver->getLinearSolver()->setMaxIterations(m_params.cg_max_iterations);
		return true;
	}
	std::shared_ptr<Math::OdeSolverEulerImplicit> getOdeSolver() const { return m_odeSolver; }

	// FemRepresentation::update(dt): one implicit-Euler step (no compliance matrix).
	void update(double dt)
	{
		if (!m_handle) throw Framework::AssertionFailure("Fem3DRepresentation::update before initialize");
		if (!m_active) return;
		detail::check(gbfem_set_solver_params(m_handle.get(), (int32_t)m_odeSolver->getNewtonRaphsonMaximumIteration(),
											  m_odeSolver->getNewtonRaphsonEpsilonConvergence(),
											  m_odeSolver->getLinearSolver()->getTolerance(),
											  m_odeSolver->getLinearSolver()->getMaxIterations()),
					  m_handle.get(), "Fem3DRepresentation::update");
		gbfem_status st = gbfem_step(m_handle.get(), dt, 1, 0);
		if (st == GBFEM_NONFINITE || st == GBFEM_INACTIVE)
		{
			m_active = false;
			return;
		}
		if (st != GBFEM_CG_MAXITER) detail::check(st, m_handle.get(), "Fem3DRepresentation::update");
	}
	// DeformableRepresentation::applyCompliance (DeformableRepresentation.cpp:175-191) and, with
	// compliance warping, FemRepresentation::applyCompliance (FemRepresentation.cpp:329-340): the
	// boundary-condition rows of b zeroed, solved with the system matrix of the last update, the
	// boundary-condition rows of the solution zeroed. `state` carries the boundary conditions in the
	// reference; here they are the body's.
	Math::Matrix applyCompliance(const Math::OdeState& state, const Math::Matrix& b)
	{
		(void)state;
		if (!m_handle) throw Framework::AssertionFailure("Ode solver not initialized, it should have been initialized on wake-up");
		int64_t n = 0, nnz = 0;
		gbfem_get_sizes(m_handle.get(), &n, &nnz);
		if (b.rows != (int32_t)n) throw Framework::AssertionFailure("applyCompliance: b has the wrong number of rows");
		Math::Matrix x(b.rows, b.cols);
		const gbfem_status st = gbfem_apply_compliance(m_handle.get(), b.cols, b.data.data(), x.data.data(),
													   m_complianceWarping ? GBFEM_COMPLIANCE_WARPING : 0u, nullptr);
		if (st != GBFEM_CG_MAXITER) detail::check(st, m_handle.get(), "applyCompliance");
		return x;
	}
	// Fem3DRepresentation::addExternalGeneralizedForce with a Fem3DLocalization (element, natural
	// coordinates): applied to the next update, then cleared. K and D are row-major 3x3 or null.
	void addExternalGeneralizedForce(int32_t element, const std::vector<double>& coordinate, const double force[3],
									 const double* K = nullptr, const double* D = nullptr)
	{
		if (!m_handle) throw Framework::AssertionFailure("addExternalGeneralizedForce before initialize");
		const size_t npe = m_params.element_type == GBFEM_ELEMENT_HEXAHEDRON ? 8 : 4;
		if (coordinate.size() != npe) throw Framework::AssertionFailure("coordinate has the wrong size");
		detail::check(gbfem_add_external_force(m_handle.get(), element, coordinate.data(), force, K, D), m_handle.get(),
					  "addExternalGeneralizedForce");
	}
	bool isActive() const { return m_active; }
	void setLocalActive(bool active)
	{
		m_active = active;
		if (active && m_handle) gbfem_reactivate(m_handle.get());
	}

	Math::OdeState getCurrentState() const
	{
		Math::OdeState s;
		int64_t n = 0, nnz = 0;
		gbfem_get_sizes(m_handle.get(), &n, &nnz);
		s.positions.resize(n);
		s.velocities.resize(n);
		detail::check(gbfem_get_state(m_handle.get(), s.positions.data(), s.velocities.data()), m_handle.get(),
					  "getCurrentState");
		return s;
	}
	void setCurrentState(const Math::OdeState& s)
	{
		detail::check(gbfem_set_state(m_handle.get(), s.positions.data(), s.velocities.data()), m_handle.get(),
					  "setCurrentState");
	}
	gbfem_handle handle() const { return m_handle.get(); }

	// Math::OdeEquation
	gbfem_handle odeHandle() const override { return m_handle.get(); }
	int32_t odeElementType() const override { return m_params.element_type; }
	gbfem_precision odePrecision() const override { return (gbfem_precision)m_params.precision; }

private:
	void checkScheme(Math::IntegrationScheme scheme) const
	{
		const bool linearElement = m_params.element_type != GBFEM_ELEMENT_COROTATIONAL_TET;
		if (scheme == Math::INTEGRATIONSCHEME_EULER_IMPLICIT) return;
		if (scheme == Math::INTEGRATIONSCHEME_LINEAR_EULER_IMPLICIT && linearElement) return;
		throw Framework::AssertionFailure(
			"unsupported integration scheme: this path steps INTEGRATIONSCHEME_EULER_IMPLICIT, or "
			"INTEGRATIONSCHEME_LINEAR_EULER_IMPLICIT with a linear element type");
	}
	struct Deleter
	{
		void operator()(gbfem_handle_s* h) const { gbfem_destroy(h); }
	};
	std::string m_name;
	std::string m_elementType = "SurgSim::Physics::Fem3DElementCorotationalTetrahedron";
	Math::IntegrationScheme m_scheme = Math::INTEGRATIONSCHEME_EULER_IMPLICIT;
	Math::LinearSolver m_linearSolver = Math::LINEARSOLVER_CONJUGATEGRADIENT;
	bool m_complianceWarping = false;
	Fem3D m_mesh;
	gbfem_params m_params{};
	std::unique_ptr<gbfem_handle_s, Deleter> m_handle;
	std::shared_ptr<Math::OdeSolverEulerImplicit> m_odeSolver;
	bool m_active = true;
};

}  // namespace Physics
}  // namespace surgsim_gb300
