// gbfem_internal.h -- shared declarations of the gbfem host code and kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gbfem {

// Per-element rest data, structure of arrays: rest[k * E + e] (FP64; the mixed form keeps an
// FP32 copy with the same layout).
//   k = 0..11  shape-function gradients g_a (a = 0..3, 3 components each) = rows of V^-1
//   k = 12     rest volume V
//   k = 13     lambda * V
//   k = 14     mu * V
//   k = 15     consistent-mass coefficient rho * V / 20
constexpr int kRestFields = 16;
// Lower-triangle blocks an element writes: 4 diagonal blocks then the 6 node pairs
// (0,1),(0,2),(0,3),(1,2),(1,3),(2,3), each stored with the larger global node id as its row.
constexpr int kSlots = 10;

// Device view of one body.
struct DevBody
{
	int N = 0, E = 0, n = 0;        // nodes, tets, dofs
	int nb = 0, nl = 0;             // blocks of the symmetric block matrix, lower blocks
	const int4* tets = nullptr;
	const double* rest = nullptr;   // kRestFields * E
	const float* rest32 = nullptr;  // FP32 copy (mixed form)
	const double* xrest = nullptr;  // 3N
	const int4* lblk = nullptr;     // nl: {I, J, SELL base of (I,J), SELL base of (J,I) or -1}
	const int* cptr = nullptr;      // nl+1
	const int* cidx = nullptr;      // E*kSlots: e*kSlots + slot, element order inside a lower block
	const double* lmass = nullptr;  // nl: consistent-mass coefficient of the lower block
	const int* iptr = nullptr;      // N+1 node incidences
	const int* iidx = nullptr;      // 4E: e*4 + a, element order
	const double* nmass = nullptr;  // N lumped node mass (gravity)
	const uint8_t* bc = nullptr;    // n boundary-condition mask
	// Mixed form, corotational: per-element rest edges q_a = x0_a - x0_0 (a = 1..3, FP32, [3(a-1)+k][E])
	// and rest Gram q_a . q_c as unevaluated float pairs hi + lo ([6][E]); per-dof inputs of the FP32
	// element kernel that its node pass writes each time it runs: x as a float pair, v, and (past the
	// first Newton iteration) x_n - x_t and v_n - v_t.
	const float* qf32 = nullptr;
	const float2* qg2 = nullptr;
	float2* nodeX = nullptr;
	float* nodeV = nullptr;
	float* nodeDx = nullptr;
	float* nodeDv = nullptr;
	int lumped = 0;                 // mass lumping (FemRepresentation::setMassLumping)
};

// Device control block of one FP64 CG solve; all scalars live on the device.
struct CgCtl
{
	double bb, rz, pq, rr, threshold, alpha, beta, pad0;
	int iter, done, converged, maxIter;
	unsigned int ticket[4];
	double newtonVar;   // max |dv - dv_prev| of the last Newton iteration
	double sumX, sumV;  // OdeState::isValid sums
	int nonfinite, pad1;
};

// Multi-right-hand-side CG (compliance columns): kMcgCols columns solved together, each with its
// own scalars and convergence test; vectors interleave the columns per dof ([i * kMcgCols + c]).
constexpr int kMcgCols = 8;
struct McgCtl
{
	double bb[kMcgCols], rz[kMcgCols], pq[kMcgCols], alpha[kMcgCols], beta[kMcgCols], rr[kMcgCols];
	double threshold[kMcgCols];
	int iter[kMcgCols], done[kMcgCols], converged[kMcgCols];
	int allDone, maxIter;
	unsigned int ticket[4];
};

struct Launch
{
	int vecGrid = 0;   // blocks of 256 threads for the dof-wise kernels
	cudaStream_t stream = nullptr;
};

// Sliced-ELL storage of the 3x3-block matrix ("SELL-32"): block rows are sorted by their number
// of blocks and cut into chunks of 32 rows; chunk c holds width[c] = off[c+1] - off[c] block
// columns. Block column k of the chunk stores, for its 32 rows (lanes), the column node id at
// col[k*32 + lane] and the 9 values (row-major inside the block) at val[k*288 + m*32 + lane].
// Rows shorter than the chunk width are padded with zero blocks pointing at the row's own node.
template <typename T>
struct MatSellT
{
	int rows;            // block rows incl. padding (a multiple of 32)
	const int* perm;     // sorted position -> node id, -1 on padding rows
	const int* off;      // chunk offsets in block columns, nchunks + 1
	const int* col;
	const T* val;
};
using MatSell3 = MatSellT<double>;
struct MatCsr
{
	int rows;
	const int* rowptr;
	const int* col;
	const double* val;
};

// ---- element / assembly
// kslots may be null (right-hand side only); linear: the linear tetrahedron (K_e = K0, no rotation).
void launch_element_fp64(const DevBody& b, const double* xn, const double* vn, const double* xt, const double* vt,
						 double dt, double alpha, double beta, double* kslots, double* rhsE, double* kfull,
						 double* fE, int* counters, cudaStream_t s, bool linear = false);
// elemsPerBlock: 32 or 64 (a tuning choice; results do not depend on it). Corotational elements
// first run the node pass (FP32 node inputs). Returns the number of kernels launched.
int launch_element_f32(const DevBody& b, const double* xn, const double* vn, const double* xt, const double* vt,
					   double dt, double alpha, double beta, float* kslots, float* rhsE, int* counters,
					   cudaStream_t s, int elemsPerBlock = 64, bool linear = false);
void launch_assemble(const DevBody& b, const double* kslots, double c1, double c2, double* A, double* invdiag,
					 cudaStream_t s);
void launch_assemble(const DevBody& b, const float* kslots, double c1, double c2, float* A, float* invdiag,
					 cudaStream_t s);
void launch_rhs_gather(const DevBody& b, const double* rhsE, const double* gravity, int gravityOn, double* rhs,
					   int applyBc, cudaStream_t s);
void launch_rhs_gather(const DevBody& b, const float* rhsE, const double* gravity, int gravityOn, double* rhs,
					   int applyBc, cudaStream_t s);
// Full (non-mirrored) system for export: CSC slots gather from full element matrices.
void launch_assemble_full_csc(int nnz, const int* sptr, const int* sidx, const int* srow, const int* scol,
							  const double* kfull, const double* smass, const uint8_t* bc, double c1, double c2,
							  double* S, cudaStream_t s);

// ---- FP64 CG on the mirrored symmetric matrix
void launch_cg_init(int n, const double* b, const double* invdiag, double* x, double* r, double* p, CgCtl* ctl,
					double* part, double tol, int maxIter, const Launch& L);
void launch_cg_spmv_sell(const MatSell3& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L);
void launch_cg_spmv_csr(const MatCsr& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L);
void launch_cg_update(int n, const double* invdiag, const double* p, const double* q, double* x, double* r,
					  CgCtl* ctl, double* part, const Launch& L);
void launch_cg_pupdate(int n, const double* invdiag, const double* r, double* p, CgCtl* ctl, const Launch& L);

// ---- state
void launch_state_update(int n, const double* dv, double* dvPrev, const double* xt, double* xn, double* vn,
						 double dt, int trackNewton, CgCtl* ctl, double* part, const Launch& L);
void launch_validity(int n, const double* x, const double* v, CgCtl* ctl, double* part, const Launch& L);
void launch_scatter_values(int count, const int* idx, const double* vals, double* dst, cudaStream_t s);
// Compliance (multi-right-hand-side CG on the stored system, compliance warping).
void launch_mcg_init(int n, int ncols, const double* B, const uint8_t* bc, const double* invd64, const float* invd32,
					 double* X, double* R, double* Z, double* P, McgCtl* ctl, double* part, double tol, int maxIter,
					 const Launch& L);
void launch_mcg_spmm(const MatSellT<double>* A64, const MatSellT<float>* A32, const double* P, double* Q,
					 McgCtl* ctl, double* part, const Launch& L);
void launch_mcg_update(int n, const double* invd64, const float* invd32, const double* P, const double* Q, double* X,
					   double* R, double* Z, McgCtl* ctl, double* part, const Launch& L);
void launch_mcg_pupdate(int n, const double* Z, double* P, const McgCtl* ctl, const Launch& L);
// Per-element rotation of the polar decomposition at positions x (9 per element, row-major).
void launch_element_rotation(const DevBody& b, const double* x, double* Re, cudaStream_t s);
// Per-node warping rotation: the running slerp average of the node's element rotations in element
// order (Fem3DCorotationalTetrahedronRepresentation.cpp:112-140).
void launch_node_rotation(const DevBody& b, const double* Re, double* Wn, cudaStream_t s);
// out = x - dt v (the positions a step started from, after x = x_t + dt v).
void launch_prev_positions(int n, const double* x, const double* v, double dt, double* out, cudaStream_t s);
// X (n x kMcgCols, interleaved) <- blockdiag(W) X, or its transpose.
void launch_apply_node_rotation(int N, const double* Wn, double* X, bool transpose, cudaStream_t s);

// Differentiation form (gbfem_adjoint.cu).
void launch_element_adjoint(const DevBody& b, const double* x, const double* v, const double* mu, const double* dv,
							double dt, double alpha, double beta, double* gx, double* gv, double* gLogE, double* gNu,
							cudaStream_t s, bool fp32 = false);
void launch_adjoint_gather(const DevBody& b, const double* gx, const double* gv, const double* lx, const double* lv,
						   double dt, double* lxOut, double* lvOut, cudaStream_t s);
void launch_adjoint_rhs(int n, const uint8_t* bc, const double* lx, const double* lv, double dt, double* g,
						cudaStream_t s);
// out = a - b (n doubles).
void launch_vec_diff(int n, const double* a, const double* b, double* out, cudaStream_t s);
void launch_set_materials(int E, const double* young, const double* poisson, double* rest, float* rest32,
						  cudaStream_t s);

// Hexahedra (gbfem_hex.cu). Element integrals once (36 lower-triangle node blocks and their scalar
// masses per element, slot order: 8 diagonal blocks, then the node pairs a < b lexicographically),
// the assembled K and scalar block masses in the SELL layout, S from them, the per-step right-hand side.
constexpr int kHexSlots = 36;
void launch_hex_element(int E, const int* nodes, const double* xrest, const double* young, const double* poisson,
						const double* rho, double* slots, double* smass, cudaStream_t s);
void launch_assemble_k(const DevBody& b, const double* slots, const double* smass, double* K, double* Ms,
					   double* lmass, cudaStream_t s);
// Mass lumping of the stored scalar block masses (Ms, both triangles) and the lower-block masses:
// row sums onto the diagonal, zero elsewhere; rowsum: N doubles of scratch.
void launch_hex_lump_masses(const DevBody& b, const MatSell3& K, double* Ms, double* lmass, double* rowsum,
							cudaStream_t s);
void launch_system_from_k(const DevBody& b, const double* K, double c1, double c2, double* A, double* invdiag,
						  cudaStream_t s);
void launch_system_from_k(const DevBody& b, const double* K, double c1, double c2, float* A, float* invdiag,
						  cudaStream_t s);
// uw: scratch of 6 doubles per node (16-byte aligned); two launches.
void launch_hex_rhs(const MatSell3& K, const double* Ms, const DevBody& b, const double* xt, const double* vn,
					const double* vt, double dt, double alpha, double beta, const double* gravity, int gravityOn,
					double* uw, double* rhs, cudaStream_t s);
// Mixed form: the same right-hand side from K and the slot masses stored as float pairs (Kp, Msp,
// launch_split_pairs), in double-float arithmetic with no FP64 in the matrix pass; same scratch.
void launch_hex_rhs_df(const MatSell3& K, const float2* Kp, const float2* Msp, const DevBody& b, const double* xt,
					   const double* vn, const double* vt, double dt, double alpha, double beta, const double* gravity,
					   int gravityOn, double* uw, double* rhs, cudaStream_t s);
// dst[i] = {hi, lo}: src[i] as an unevaluated float pair (hi = src rounded, lo = the rest rounded).
void launch_split_pairs(size_t n, const double* src, float2* dst, cudaStream_t s);

// External generalized forces of one step (Fem3DRepresentation::addExternalGeneralizedForce):
// updates of lower system blocks (I >= J; z/w the SELL bases of (I,J) and (J,I), w < 0 on the
// diagonal) with D + dt K, and right-hand-side rows with F + sum_J K_IJ (x_n - x_t - dt v_n)_J.
struct ExtBlock
{
	int z, w, I, J;
	double v[9];
};
struct ExtRow
{
	int I, k0, k1, pad;
	double F[3];
};
struct ExtCol
{
	int J, pad;
	double K[9];
};
void launch_ext_system(int count, const ExtBlock* blocks, const uint8_t* bc, double* A, double* invdiag, cudaStream_t s);
void launch_ext_system(int count, const ExtBlock* blocks, const uint8_t* bc, float* A, float* invdiag, cudaStream_t s);
void launch_ext_rhs(int count, const ExtRow* rows, const ExtCol* cols, const uint8_t* bc, const double* xn,
					const double* xt, const double* vn, double dt, double* rhs, cudaStream_t s);

// Partial-sum buffer size needed by the reductions for a given vecGrid.
constexpr int partial_slots(int vecGrid) { return 4 * (vecGrid + 1024); }

}  // namespace gbfem
