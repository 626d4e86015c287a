/*
 * gbfem.h -- C ABI of the GB300 (sm_103a) corotational-tetrahedron FEM implicit-Euler step.
 *
 * One handle is one deformable body: OpenSurgSim's Fem3DRepresentation with
 * Fem3DElementCorotationalTetrahedron elements, IntegrationScheme EULER_IMPLICIT and
 * LinearSolver CONJUGATEGRADIENT. All device memory belongs to the handle; every array passed in
 * is copied during the call. No function throws; every function returns a gbfem_status and the
 * message of the last failure is available from gbfem_last_error.
 *
 * Threading matches the reference's FreeMotion: one handle is used by one thread at a time;
 * different handles may be used concurrently (each has its own CUDA stream).
 *
 * Reference interfaces replaced (paths inside the OpenSurgSim tree):
 *   SurgSim/Physics/Fem3DRepresentation.h        setFem/loadFem, setInitialState, initialize
 *   SurgSim/Physics/FemRepresentation.cpp:232-294 update(dt)
 *   SurgSim/Math/OdeSolverEulerImplicit.h:33-76    solve, setNewtonRaphson*
 *   SurgSim/Math/LinearSparseSolveAndInverse.h:98-123  LinearSparseSolveAndInverseCG
 *   SurgSim/Math/OdeState.h:38-207                 positions, velocities, boundary conditions
 */
#ifndef GBFEM_H
#define GBFEM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBFEM_API __attribute__((visibility("default")))
#else
#define GBFEM_API
#endif

/* Status codes. The reference throws SurgSim::Framework::AssertionFailure for invalid input
 * (Framework/Assert.h:77-95) and deactivates a representation whose state is not finite
 * (FemRepresentation.cpp:285-293); these codes carry the same outcomes across the ABI. */
typedef enum gbfem_status
{
	GBFEM_OK = 0,
	GBFEM_INVALID_ARG = 1,          /* bad sizes, indices, materials or parameters */
	GBFEM_DEGENERATE_ELEMENT = 2,   /* rest tetrahedron not invertible (|det V| <= 1e-12) */
	GBFEM_CG_MAXITER = 3,           /* CG stopped at maxIterations; the step was still applied */
	GBFEM_NONFINITE = 4,            /* state became NaN/Inf; the handle is deactivated */
	GBFEM_CUDA_ERROR = 5,
	GBFEM_INACTIVE = 6,             /* step called on a deactivated handle: no-op */
	GBFEM_OUT_OF_MEMORY = 7
} gbfem_status;

/* Arithmetic of the step. */
typedef enum gbfem_precision
{
	GBFEM_PRECISION_FP64 = 0,   /* plain form: FP64 throughout */
	GBFEM_PRECISION_MIXED = 1   /* FP32 element kernels and CG, FP64 iterative refinement */
} gbfem_precision;

typedef struct gbfem_handle_s* gbfem_handle;

/* Mesh: Fem3DRepresentation::setFem (Fem3DRepresentation.cpp:70-126) + per-element material
 * (FemElement3DParameter) + OdeState boundary conditions (OdeState.cpp:115-142). */
typedef struct gbfem_mesh_desc
{
	int32_t num_nodes;
	const double* rest_positions;   /* [3 * num_nodes], node-major x,y,z */
	int32_t num_tets;               /* elements (tetrahedra, or hexahedra for GBFEM_ELEMENT_HEXAHEDRON) */
	const int32_t* tets;            /* [4 * num_tets] node ids; [8 * num_tets] for hexahedra */
	const double* young_modulus;    /* [num_tets] */
	const double* poisson_ratio;    /* [num_tets] */
	const double* mass_density;     /* [num_tets] */
	int32_t num_bc_dofs;
	const int32_t* bc_dofs;         /* dof ids 3*node+axis; duplicates are ignored */
} gbfem_mesh_desc;

typedef struct gbfem_params
{
	double rayleigh_mass;           /* FemRepresentation RayleighDampingMass (alpha) */
	double rayleigh_stiffness;      /* FemRepresentation RayleighDampingStiffness (beta) */
	double gravity[3];              /* Representation.cpp:36 default (0, -9.81, 0) */
	int32_t gravity_enabled;
	int32_t newton_max_iterations;  /* OdeSolverEulerImplicit default 1 */
	double newton_epsilon;          /* default 1e-5 (infinity norm of the solution variation) */
	double cg_tolerance;            /* LinearSparseSolveAndInverseCG::setTolerance */
	int32_t cg_max_iterations;      /* setMaxIterations; <= 0 selects Eigen's default 2n (mixed form: 2n + 64,
	                                   FP32 CG needs up to ~2.5n iterations on systems of a few tens of dofs;
	                                   in a batch, n is each mesh's own dof count) */
	int32_t precision;              /* gbfem_precision */
	int32_t device;                 /* CUDA device ordinal */
	int32_t autotune;               /* mixed form: tune block sizes and the solve schedule on the first step */
	int32_t element_type;           /* GBFEM_ELEMENT_COROTATIONAL_TET (default), _LINEAR_TET or _HEXAHEDRON */
	int32_t mass_lumping;           /* FemRepresentation::setMassLumping (FemRepresentation.cpp:320-323): 1 sums
	                                   every row of M onto its diagonal (:499-508) for the system matrix, the
	                                   Rayleigh mass force (:584-586) and the Newton mass term; default 0 */
	int32_t reserved[4];
} gbfem_params;

/* Per-call statistics of the last gbfem_step. */
typedef struct gbfem_stats
{
	int32_t steps;                  /* steps applied */
	int32_t cg_iterations;          /* summed over steps and Newton iterations (Eigen's count) */
	int32_t cg_max_iterations_hit;  /* number of solves that stopped at maxIterations */
	int32_t refinement_sweeps;      /* mixed precision: true-residual evaluations (refreshes) */
	double cg_relative_residual;    /* of the last solve: sqrt(|r|^2/|b|^2) */
	double ms_element, ms_assemble, ms_solve, ms_update;  /* device time per phase (if timed) */
	int32_t singular_g;             /* element updates that hit the singular-G early return */
	int32_t polar_fallbacks;        /* element updates that took the SVD polar path */
	int32_t active;
	int32_t kernel_launches;        /* kernels this call launched */
	int32_t spmv_timed;             /* CG matrix-vector launches timed (GBFEM_STEP_TIME_KERNELS) */
	int32_t reserved0;
	double ms_spmv;                 /* summed device time of those launches (CUDA events) */
	double reserved[2];
} gbfem_stats;

/* Element types (gbfem_params.element_type).
 *  COROTATIONAL_TET: Fem3DElementCorotationalTetrahedron (Fem3DElementCorotationalTetrahedron.cpp:77-288)
 *                    stepped by OdeSolverEulerImplicit.
 *  LINEAR_TET:       Fem3DElementTetrahedron (Fem3DElementTetrahedron.cpp:77-90: K_e = K0,
 *                    f_e = -K0 (x - x0)) stepped by OdeSolverLinearEulerImplicit
 *                    (OdeSolverLinearEulerImplicit.cpp:43-64): the first step assembles and solves the
 *                    full system; later steps (same dt and materials) update only the right-hand side
 *                    and solve with the stored system matrix. The dense compliance matrix the reference
 *                    forms on the first step is not formed (every solve is a CG solve).
 *  HEXAHEDRON:       Fem3DElementCube (Fem3DElementCube.cpp:65-141): 8 nodes per element in the order
 *                    of its shape-function signs (eps, eta, mu) = (-,-,-) (+,-,-) (+,+,-) (-,+,-)
 *                    (-,-,+) (+,-,+) (+,+,+) (-,+,+); K and M by 2x2x2 Gauss-Legendre quadrature at the
 *                    rest state, f = -K (x - x0). A linear element: K and M are computed and assembled
 *                    once on the device, S = (1/dt + alpha) M + (dt + beta) K is formed again only when dt
 *                    or a material changes, and each step forms its right-hand side in one pass over the
 *                    stored K and M. gbfem_create fails with GBFEM_DEGENERATE_ELEMENT where the
 *                    reference's initialize asserts (a Jacobian with |det| <= 1e-12 at a Gauss point, or a
 *                    rest volume <= 1e-12). */
#define GBFEM_ELEMENT_COROTATIONAL_TET 0
#define GBFEM_ELEMENT_LINEAR_TET 1
#define GBFEM_ELEMENT_HEXAHEDRON 2

/* Flags for gbfem_step. */
#define GBFEM_STEP_TIME_PHASES 1u   /* record per-phase device times (adds events) */
#define GBFEM_STEP_KEEP_SYSTEM 2u   /* keep the full S / rhs / f of the last solve for export */
#define GBFEM_STEP_TIME_KERNELS 4u  /* time every CG matrix-vector launch with CUDA events */
#define GBFEM_STEP_GRAPH 8u         /* mixed form or batch, one Newton iteration: capture the step into a CUDA graph
                                       once and launch it nsteps times with no host round trip between
                                       steps (statistics and the finiteness check are read at the end,
                                       so a non-finite state is reported after the last step) */

GBFEM_API gbfem_status gbfem_params_default(gbfem_params* out);

/* Build a body: copies the mesh, precomputes rest quantities (Fem3DElementTetrahedron.cpp:92-216,
 * Fem3DElementCorotationalTetrahedron.cpp:48-75), the sparsity pattern and the element-to-nonzero
 * maps (FemRepresentation.cpp:85-132). The state starts at rest with zero velocity. */
GBFEM_API gbfem_status gbfem_create(const gbfem_mesh_desc* mesh, const gbfem_params* params, gbfem_handle* out);
GBFEM_API gbfem_status gbfem_destroy(gbfem_handle h);

/* FemRepresentation::update(dt) repeated nsteps times (OdeSolverEulerImplicit::solve with
 * computeCompliance = false). Returns GBFEM_NONFINITE (and deactivates) when the state stops being
 * finite, GBFEM_CG_MAXITER when a solve hit maxIterations, GBFEM_INACTIVE when deactivated. */
GBFEM_API gbfem_status gbfem_step(gbfem_handle h, double dt, int32_t nsteps, uint32_t flags);
GBFEM_API gbfem_status gbfem_get_stats(gbfem_handle h, gbfem_stats* out);

/* OdeState positions / velocities, host arrays of 3*num_nodes doubles (either may be NULL). */
GBFEM_API gbfem_status gbfem_get_state(gbfem_handle h, double* x, double* v);
GBFEM_API gbfem_status gbfem_set_state(gbfem_handle h, const double* x, const double* v);
/* v[dofs[i]] = values[i]: prescribe the velocity of (boundary-condition) dofs before a step. */
GBFEM_API gbfem_status gbfem_set_velocities(gbfem_handle h, int32_t count, const int32_t* dofs,
											const double* values);
/* Same with dofs and values already in device memory of the handle's GPU (no host copy). */
GBFEM_API gbfem_status gbfem_set_velocities_device(gbfem_handle h, int32_t count, const int32_t* dofs_dev,
												   const double* values_dev);
/* Device pointers of the state (FP64, 3*num_nodes each), valid until gbfem_destroy. */
GBFEM_API gbfem_status gbfem_device_state(gbfem_handle h, double** x, double** v);
/* The CUDA stream the handle launches on (a cudaStream_t). */
GBFEM_API gbfem_status gbfem_stream(gbfem_handle h, void** stream);
GBFEM_API gbfem_status gbfem_reactivate(gbfem_handle h);

/* ---- Compliance (DeformableRepresentation::applyCompliance, DeformableRepresentation.cpp:175-191;
 * with warping, FemRepresentation::applyCompliance, FemRepresentation.cpp:329-340, and the node
 * rotations of Fem3DCorotationalTetrahedronRepresentation.cpp:85-143). For each of the ncols columns of b
 * (host, column-major n x ncols, e.g. constraint directions): zero the boundary-condition rows, solve
 * with the system matrix of the last step, zero the boundary-condition rows of the solution, write the
 * column of x. The columns are solved together, eight at a time, by a multi-right-hand-side CG that
 * reads the matrix once per iteration for all of them; each column has its own Eigen-style
 * convergence test (tolerance and maximum iterations of the handle). Replaces the dense inverse the
 * reference forms for getComplianceMatrix(); the dense matrix is this call on the identity's
 * columns. GBFEM_COMPLIANCE_WARPING: x = W S^-1 W^T b with W the per-node slerp average of the element
 * rotations at the positions the last step started from (corotational element only). iterations
 * (may be NULL) receives the CG iterations summed over columns. Returns GBFEM_CG_MAXITER if a column
 * did not converge. */
#define GBFEM_COMPLIANCE_WARPING 1u
GBFEM_API gbfem_status gbfem_apply_compliance(gbfem_handle h, int32_t ncols, const double* b, double* x, uint32_t flags,
											  int32_t* iterations);

/* Fem3DRepresentation::addExternalGeneralizedForce (Fem3DRepresentation.cpp:133-197) with a
 * Fem3DLocalization: a force `force` (3) at the point of element `element` with natural (barycentric)
 * coordinates coord[4] (coord[8] for hexahedra), and an optional 3x3 stiffness and damping (row-major;
 * NULL for none). Element node a receives coord[a] * force and node pair (a, b) coord[a] coord[b] *
 * stiffness / damping. Calls accumulate; the next gbfem_step applies them to its first step
 * (FemRepresentation::computeFMDK, FemRepresentation.cpp:527-544: f += F, K += K_ext, D += D_ext, in
 * every Newton iteration of that step) and then clears them (DeformableRepresentation::afterUpdate,
 * DeformableRepresentation.cpp:242-252). Element ids of a batch handle run over the concatenated
 * meshes. The adjoint step does not see them. */
GBFEM_API gbfem_status gbfem_add_external_force(gbfem_handle h, int32_t element, const double* coord, const double* force,
												const double* stiffness, const double* damping);

/* Solver settings after creation: OdeSolverEulerImplicit::setNewtonRaphsonMaximumIteration /
 * setNewtonRaphsonEpsilonConvergence (OdeSolverEulerImplicit.cpp:31-53) and
 * LinearSparseSolveAndInverseCG::setTolerance / setMaxIterations (LinearSparseSolveAndInverse.cpp:99-117),
 * which the reference allows at any time; they take effect at the next step (a captured step graph
 * is captured again). newton_max_iterations >= 1; cg_max_iterations <= 0 selects the default cap. */
GBFEM_API gbfem_status gbfem_set_solver_params(gbfem_handle h, int32_t newton_max_iterations, double newton_epsilon,
											   double cg_tolerance, int32_t cg_max_iterations);

/* ---- Tuning of the mixed form (no counterpart in the reference). With params.autotune the first
 * step times the element kernel at 32 and 64 elements per block and the persistent solve in each CG
 * schedule at 2, 3, 4 CTAs per SM and refresh weights 1 to 4 on its own system, and keeps the
 * fastest. The solve's schedule and partition set the rounding of its sums, so a run that must
 * repeat another bit for bit reads the choice with gbfem_get_tuning and pins it with
 * gbfem_set_tuning (which also disables autotune).
 * CG schedules of the persistent solve (the iteration the mixed form runs; results agree to the
 * solve's tolerance, not bit for bit; both stop by the same rule on the same FP64 residual):
 *   GBFEM_CG_TWO_PHASE: two grid-wide phases an iteration (SpMV with p.Ap; then the row update
 *     with r.z), the textbook PCG recurrences;
 *   GBFEM_CG_ONE_PHASE: one phase an iteration (Chronopoulos and Gear's recurrences, both dot
 *     products from one reduction): half the phases, larger neighbour records;
 *   GBFEM_CG_FP64: FP64 batches (their only schedule).
 * Without autotuning a handle starts in GBFEM_CG_ONE_PHASE when its system has at most 64 chunks of
 * 32 rows per SM (a few per warp: phases wait on latency), else in GBFEM_CG_TWO_PHASE.
 * gbfem_set_tuning's cg_schedule -1 keeps the handle's current schedule. */
#define GBFEM_CG_TWO_PHASE 0
#define GBFEM_CG_FP64 1
#define GBFEM_CG_ONE_PHASE 2
GBFEM_API gbfem_status gbfem_get_tuning(gbfem_handle h, int32_t* elems_per_block, int32_t* ctas_per_sm,
										int32_t* refresh_weight, int32_t* cg_schedule);
GBFEM_API gbfem_status gbfem_set_tuning(gbfem_handle h, int32_t elems_per_block, int32_t ctas_per_sm,
										int32_t refresh_weight, int32_t cg_schedule);

/* ---- Differentiation form. No counterpart in the reference (it has no adjoint); these serve
 * gradient-based identification on the same step (opensurgsim_gb300.autograd).
 *
 * Per-element moduli from device arrays (E_e, and nu_e or NULL to keep each element's current nu):
 * the reference sets them per element through Fem3DElementTetrahedron::setYoungModulus /
 * setPoissonRatio before initialize (Fem3DElementTetrahedron.h); here they can change between
 * steps. */
GBFEM_API gbfem_status gbfem_set_materials_device(gbfem_handle h, const double* young, const double* poisson);
/* Reverse-mode derivative of one gbfem_step(h, dt, 1, 0) taken from state (x, v) with velocity
 * increment dv = v' - v: given lx = dL/dx' and lv = dL/dv', writes lx_out = dL/dx and
 * lv_out = dL/dv (may alias lx / lv) and adds dL/d(log E_e) and dL/d(nu_e) into grad_log_young and
 * grad_poisson (either may be NULL). One Newton iteration (the reference default). All pointers are
 * device arrays of n (state) or num_tets (gradients) doubles. Rebuilds the step's system at (x, v)
 * and solves it transposed with the handle's CG (the FP64 or the mixed solver); the element
 * derivatives run in the handle's element precision (FP64, or FP32 for the mixed form). Does not
 * change the handle's state. Returns GBFEM_CG_MAXITER if the transposed solve did not converge
 * (the outputs are still written). Corotational elements only. With GBFEM_STEP_TIME_PHASES in flags
 * the call adds its device times to the stats: ms_element (system rebuild), ms_solve (transposed
 * solve), ms_update (element derivatives and the node gather). */
GBFEM_API gbfem_status gbfem_adjoint_step(gbfem_handle h, double dt, const double* x, const double* v, const double* dv,
										  const double* lx, const double* lv, double* lx_out, double* lv_out,
										  double* grad_log_young, double* grad_poisson, uint32_t flags);

/* Whole rollouts of the differentiation form as CUDA graphs (corotational elements, the mixed form
 * or a batch, one Newton iteration). No counterpart in the reference.
 * gbfem_rollout_forward: from (x0, v0) take nsteps steps of dt (gbfem_step semantics), keeping the
 *   state every checkpoint_every steps in device memory of the handle; writes the final state to
 *   (xT, vT) and leaves it as the handle's state.
 * gbfem_rollout_backward: the reverse sweep of the last forward: for each checkpoint segment, last
 *   first, its steps are run again from the checkpoint to recover their states, then the step
 *   adjoints (gbfem_adjoint_step) are applied in reverse. With checkpoint_every = 1 the forward keeps
 *   every state (2n doubles a step) and no step is run again. Given (lxT, lvT) = dL/d(xT, vT) it writes
 *   (lx0, lv0) = dL/d(x0, v0) and, where not NULL, grad_log_young = dL/d(log E_e) and grad_poisson =
 *   dL/d(nu_e) (overwritten, not accumulated). The handle's state is the forward's final state again
 *   afterwards.
 * Each is captured once into one CUDA graph (again when dt, nsteps, checkpoint_every or the tuning
 * changes) and launched with no host round trip inside it; the call copies its arrays in and out
 * around the launch and reads the solves' statistics once at the end. All arrays are device arrays of
 * n (state) or num_tets (gradients) doubles. Returns GBFEM_CG_MAXITER when a solve did not converge
 * (the outputs are still written) and GBFEM_NONFINITE when a forward state stopped being finite.
 * With autotune, the first forward tunes the solve on (x0, v0) before capturing. */
GBFEM_API gbfem_status gbfem_rollout_forward(gbfem_handle h, double dt, int32_t nsteps, int32_t checkpoint_every,
											 const double* x0, const double* v0, double* xT, double* vT);
GBFEM_API gbfem_status gbfem_rollout_backward(gbfem_handle h, const double* lxT, const double* lvT, double* lx0,
											  double* lv0, double* grad_log_young, double* grad_poisson);

/* ---- Batching: many independent meshes (each its own OpenSurgSim representation, stepped like
 * one FreeMotion pass over them, FreeMotion.cpp:55-80) in one body. Node ids, boundary-condition
 * dofs and states are concatenated in mesh order; every mesh keeps its own CG scalars and
 * convergence test, and one persistent launch solves all of them: in the mixed form its FP32 CG with
 * FP64 refreshes; in the FP64 form (GBFEM_PRECISION_FP64) every mesh's Eigen CG in FP64 (the same
 * iteration and stopping rule as a single FP64 handle, which solves with separate launches per
 * iteration), after the FP64 element update and assembly. Both take GBFEM_STEP_GRAPH and the
 * autotuner (CTAs per SM of the solve). gbfem_step, gbfem_get_state, gbfem_set_velocities ... act on
 * the batch. */
GBFEM_API gbfem_status gbfem_batch_create(int32_t count, const gbfem_mesh_desc* meshes, const gbfem_params* params,
										  gbfem_handle* out);
/* Number of meshes, their node / tet offsets (count + 1 entries each) and the scalar non-zeros of
 * each mesh's system matrix (count entries) in the batch. Any pointer may be NULL. */
GBFEM_API gbfem_status gbfem_batch_info(gbfem_handle h, int32_t* count, int32_t* node_offsets,
										int32_t* tet_offsets, int64_t* nnz_per_mesh);
/* Per mesh, over the last gbfem_step call: CG iterations, true-residual refreshes, converged (all
 * steps), worst relative residual. Arrays of `count` entries (any may be NULL). */
GBFEM_API gbfem_status gbfem_batch_segment_stats(gbfem_handle h, int32_t* iterations, int32_t* refreshes,
												 int32_t* converged, double* relative_residual);

/* Sizes: dofs n = 3*num_nodes, scalar nonzeros of the pattern. */
GBFEM_API gbfem_status gbfem_get_sizes(gbfem_handle h, int64_t* num_dofs, int64_t* nnz);
/* Global pattern in CSC (Eigen ColMajor, int StorageIndex): colptr[n+1], rowidx[nnz], rows sorted.
 * The pattern is structurally symmetric, so these are also the CSR arrays. */
GBFEM_API gbfem_status gbfem_get_pattern(gbfem_handle h, int32_t* colptr, int32_t* rowidx);
/* Element-to-nonzero map: map[e*D*D + (3a+i)*D + 3b+j] = CSC slot of global entry
 * (3*tet[e][a]+i, 3*tet[e][b]+j) -- the slots FemElement::assembleMatrixBlocksNoInitialize writes;
 * D = 12 for tetrahedra, 24 for hexahedra. */
GBFEM_API gbfem_status gbfem_get_scatter(gbfem_handle h, int32_t* map);
/* System of the last solve (requires GBFEM_STEP_KEEP_SYSTEM on that step): S values in CSC order
 * with boundary conditions applied (full, not mirrored), rhs[n], and the force vector f[n]. */
GBFEM_API gbfem_status gbfem_get_system(gbfem_handle h, double* S_csc, double* rhs, double* f);

/* Human-readable message of the last failure on h (or of the last failed create when h is NULL). */
GBFEM_API gbfem_status gbfem_last_error(gbfem_handle h, char* buf, size_t len);

/* Self-test of the bounded wait of the batched solve's grid barrier. No counterpart in the
 * reference (its solve runs on one CPU thread and never waits on another). The mixed-precision
 * solve is one cooperative launch whose blocks wait for one another at a grid barrier every
 * phase; each wait gives up after a wall-time limit (1 s in the solve), records an error, and the
 * step returns GBFEM_CUDA_ERROR instead of hanging. This runs that same barrier code on the current
 * device, without a handle, in one cooperative block per SM, for `phases` barriers.
 *   stall == 0: a plain run; GBFEM_OK once every block passed every barrier.
 *   stall != 0: the barrier's arrival counter starts past its last arrival, so no block is ever
 *     released (a flag that nothing sets): every wait must run out after timeout_ns, and the call
 *     returns GBFEM_CUDA_ERROR, the status a solve whose barrier timed out reports. The CUDA
 *     context stays usable.
 * timeout_ns in [1000, 2e9]; phases in [1, 1e6]. *phases_passed (may be NULL) = fewest barriers a
 * block passed; *max_wait_ns (may be NULL) = longest time a block spent in the kernel. */
GBFEM_API gbfem_status gbfem_barrier_selftest(int32_t phases, int32_t stall, int64_t timeout_ns,
											  int32_t* phases_passed, int64_t* max_wait_ns);

/* ---- LinearSparseSolveAndInverseCG on a caller matrix (LinearSparseSolveAndInverse.cpp:99-129).
 * Jacobi-preconditioned CG reading only the lower triangle (row >= col) of the CSC matrix, zero
 * initial guess, stop when |r|^2 < max(tol^2 |b|^2, DBL_MIN) or after max_iterations
 * (<= 0: 2n). Host arrays in, host solution out. */
typedef struct gbfem_cg_s* gbfem_cg;
GBFEM_API gbfem_status gbfem_cg_create(int32_t n, const int32_t* colptr, const int32_t* rowidx,
									   const double* values, int32_t device, gbfem_cg* out);
GBFEM_API gbfem_status gbfem_cg_set_tolerance(gbfem_cg cg, double tolerance);
GBFEM_API gbfem_status gbfem_cg_set_max_iterations(gbfem_cg cg, int32_t max_iterations);
GBFEM_API gbfem_status gbfem_cg_solve(gbfem_cg cg, const double* b, double* x, int32_t* iterations,
									  double* relative_residual);
GBFEM_API gbfem_status gbfem_cg_destroy(gbfem_cg cg);

/* ---- The same Jacobi-PCG solve for callers that must not allocate memory.
 * No counterpart in the reference. Some callers cannot call cudaMalloc once they are running: the
 * fixed-rate physics and haptics loops of a surgical simulator (where an allocator call can block
 * or synchronise the device at an unpredictable moment) and hosts that reserve all device memory
 * at start-up. This entry point takes the matrix and vectors already in device memory and uses a
 * scratch area that is part of the loaded library (a fixed array in device memory, on every GPU
 * that loads the library, kept until the process exits), so it makes no cudaMalloc, cudaFree,
 * pinned-memory or other allocating call.
 *   rowptr[n+1], col[nnz], values[nnz]: the full symmetric matrix in CSR form, device pointers
 *   b[n] (in), x[n] (out): device pointers;  stream: a cudaStream_t (NULL: default stream)
 * The solve is the one gbfem_cg_solve runs (zero initial guess, Jacobi preconditioner, stop when
 * |r|^2 < max(tol^2 |b|^2, DBL_MIN) or after max_iterations, <= 0 meaning 2n).
 * Limits: n <= GBFEM_NOALLOC_MAX_DOFS, else GBFEM_INVALID_ARG (message from gbfem_last_error(NULL)).
 * The matrix is checked on the device before the solve reads through it: rowptr[0] != 0, a
 * decreasing rowptr or a column index outside [0, n) returns GBFEM_INVALID_ARG (the message names
 * the first bad row); rowptr must hold n + 1 entries and col / values rowptr[n] each.
 * The first call in a context of a device (the first call on the device, and the first after the
 * device was reset) looks up the scratch area's device address with that device current; make that
 * first call before any stream capture. Each call waits for its stream: it reads the solve's
 * control block back to the host between batches of iterations. Every call shares the one scratch
 * area, which keeps the last call's contents (each call clears what must start at zero): calls
 * that overlap on the same GPU race and must be serialised by the caller. */
#define GBFEM_NOALLOC_MAX_DOFS 262144
GBFEM_API gbfem_status gbfem_cg_solve_noalloc(int32_t n, const int32_t* rowptr, const int32_t* col,
											  const double* values, const double* b, double* x, double tolerance,
											  int32_t max_iterations, void* stream, int32_t* iterations,
											  double* relative_residual);

#ifdef __cplusplus
}
#endif

#endif /* GBFEM_H */
