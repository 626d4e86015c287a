// surgsim_gb300.h -- header-only C++ facade over the gbfem C ABI that keeps OpenSurgSim's class and
// method names for the corotational-tetrahedron implicit-Euler path, so code written against
//   SurgSim::Physics::Fem3DRepresentation   (Physics/Fem3DRepresentation.h, FemRepresentation.h,
//                                            DeformableRepresentation.h)
//   SurgSim::Math::OdeSolverEulerImplicit   (Math/OdeSolverEulerImplicit.h)
//   SurgSim::Math::LinearSparseSolveAndInverseCG (Math/LinearSparseSolveAndInverse.h:98-123)
// can switch to the GB300 step by changing the namespace. Failures throw AssertionFailure (the
// reference's SurgSim::Framework::AssertionFailure, Framework/Assert.h:77-95) carrying the
// message of gbfem_last_error; a representation whose state stops being finite is deactivated
// instead, as in FemRepresentation::update (FemRepresentation.cpp:285-293).
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

enum IntegrationScheme
{
	INTEGRATIONSCHEME_EULER_IMPLICIT = 2  // the only scheme of this path (MathConvert.h names)
};
enum LinearSolver
{
	LINEARSOLVER_CONJUGATEGRADIENT = 1
};

// Positions and velocities of a representation (Math/OdeState.h), node-major x,y,z.
struct OdeState
{
	std::vector<double> positions, velocities;
	const std::vector<double>& getPositions() const { return positions; }
	const std::vector<double>& getVelocities() const { return velocities; }
	size_t getNumDof() const { return positions.size(); }
	size_t getNumNodes() const { return positions.size() / 3; }
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

class Fem3DRepresentation
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
		if (type == "SurgSim::Physics::Fem3DElementCorotationalTetrahedron")
			m_params.element_type = GBFEM_ELEMENT_COROTATIONAL_TET;
		else if (type == "SurgSim::Physics::Fem3DElementTetrahedron")
			m_params.element_type = GBFEM_ELEMENT_LINEAR_TET;
		else if (type == "SurgSim::Physics::Fem3DElementCube")
			m_params.element_type = GBFEM_ELEMENT_HEXAHEDRON;
		else
			throw Framework::AssertionFailure("unsupported element type " + type);
		m_elementType = type;
	}
	const std::string& getFemElementType() const { return m_elementType; }
	void setIntegrationScheme(Math::IntegrationScheme) {}
	void setLinearSolver(Math::LinearSolver) {}
	void setRayleighDampingMass(double c) { m_params.rayleigh_mass = c; }
	void setRayleighDampingStiffness(double c) { m_params.rayleigh_stiffness = c; }
	void setIsGravityEnabled(bool on) { m_params.gravity_enabled = on ? 1 : 0; }
	// The reference's gravity is fixed at (0, -9.81, 0) (Representation.cpp:36); this one can be set.
	void setGravity(double gx, double gy, double gz)
	{
		m_params.gravity[0] = gx;
		m_params.gravity[1] = gy;
		m_params.gravity[2] = gz;
	}
	// OdeSolverEulerImplicit settings (OdeSolverEulerImplicit.cpp:31-53).
	void setNewtonRaphsonMaximumIteration(int32_t n)
	{
		if (n < 1) throw Framework::AssertionFailure("The maximum iteration needs to be at least 1");
		m_params.newton_max_iterations = n;
	}
	void setNewtonRaphsonEpsilonConvergence(double eps)
	{
		if (eps < 0) throw Framework::AssertionFailure("The epsilon convergence cannot be negative");
		m_params.newton_epsilon = eps;
	}
	// LinearSparseSolveAndInverseCG settings.
	void setLinearSolverTolerance(double tol) { m_params.cg_tolerance = tol; }
	void setLinearSolverMaxIterations(int32_t it) { m_params.cg_max_iterations = it; }
	// GB300 extension: FP64 plain form or FP32 with FP64 refinement.
	void setPrecision(gbfem_precision p) { m_params.precision = p; }
	void setDevice(int32_t device) { m_params.device = device; }

	// Representation::initialize + wakeUp: builds the device body.
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
		return true;
	}

	// FemRepresentation::update(dt): one implicit-Euler step (no compliance matrix).
	void update(double dt)
	{
		if (!m_handle) throw Framework::AssertionFailure("Fem3DRepresentation::update before initialize");
		if (!m_active) return;
		gbfem_status st = gbfem_step(m_handle.get(), dt, 1, 0);
		if (st == GBFEM_NONFINITE || st == GBFEM_INACTIVE)
		{
			m_active = false;
			return;
		}
		if (st != GBFEM_CG_MAXITER) detail::check(st, m_handle.get(), "Fem3DRepresentation::update");
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

private:
	struct Deleter
	{
		void operator()(gbfem_handle_s* h) const { gbfem_destroy(h); }
	};
	std::string m_name;
	std::string m_elementType = "SurgSim::Physics::Fem3DElementCorotationalTetrahedron";
	Fem3D m_mesh;
	gbfem_params m_params{};
	std::unique_ptr<gbfem_handle_s, Deleter> m_handle;
	bool m_active = true;
};

}  // namespace Physics
}  // namespace surgsim_gb300
