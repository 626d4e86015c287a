// gbfem_host.cpp -- host side of the gbfem C ABI: validation, rest precompute, sparsity pattern
// and element-to-nonzero maps, step orchestration on the handle's CUDA stream.

#include <algorithm>
#include <array>
#include <map>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gbfem.h"
#include "gbfem_internal.h"
#include "gbfem_pcg.h"

using namespace gbfem;

static_assert(GBFEM_CG_TWO_PHASE == kPcgMixed2 && GBFEM_CG_FP64 == kPcgF64 && GBFEM_CG_ONE_PHASE == kPcgMixed1,
			  "the ABI's CG schedules are the persistent solve's forms");

namespace {

thread_local std::string g_lastCreateError;

template <typename T>
struct DevBuf
{
	T* p = nullptr;
	size_t n = 0;
	cudaError_t alloc(size_t count)
	{
		free();
		n = count;
		if (count == 0) return cudaSuccess;
		return cudaMalloc(&p, count * sizeof(T));
	}
	cudaError_t upload(const T* src, size_t count, cudaStream_t s)
	{
		cudaError_t e = alloc(count);
		if (e != cudaSuccess || count == 0) return e;
		return cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s);
	}
	void free()
	{
		if (p) cudaFree(p);
		p = nullptr;
		n = 0;
	}
};

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

// Inverse of the 4x4 homogeneous rest matrix with the |det| > 1e-12 check of
// Fem3DElementCorotationalTetrahedron.cpp:57-72.
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

// Rest checks of Fem3DElementCube::initialize: the Jacobian at each of the 8 Gauss points must be
// invertible (|det J| > 1e-12, Fem3DElementCube.cpp:202-207) and the rest volume, the sum of the
// determinants (weights 1, :321-366), above 1e-12 (:357). Returns 0, 1 (singular J) or 2 (volume).
int hex_rest_check(const double* X, const int32_t* nd, double* volume)
{
	static const double sE[8] = {-1, 1, 1, -1, -1, 1, 1, -1}, sH[8] = {-1, -1, 1, 1, -1, -1, 1, 1},
						sM[8] = {-1, -1, -1, -1, 1, 1, 1, 1};
	const double q = 1.0 / std::sqrt(3.0);
	double v = 0.0;
	for (int gp = 0; gp < 8; ++gp)
	{
		const double e = (gp & 4) ? -q : q, h = (gp & 2) ? -q : q, m = (gp & 1) ? -q : q;
		double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
		for (int i = 0; i < 8; ++i)
		{
			const double d[3] = {0.125 * sE[i] * (1 + h * sH[i]) * (1 + m * sM[i]),
								 0.125 * (1 + e * sE[i]) * sH[i] * (1 + m * sM[i]),
								 0.125 * (1 + e * sE[i]) * (1 + h * sH[i]) * sM[i]};
			for (int r = 0; r < 3; ++r)
				for (int c = 0; c < 3; ++c) J[r][c] += X[3 * (size_t)nd[i] + c] * d[r];
		}
		const double det = det33(J);
		if (!(std::fabs(det) > 1e-12)) return 1;
		v += det;
	}
	*volume = v;
	return v > 1e-12 ? 0 : 2;
}

}  // namespace

struct gbfem_handle_s
{
	int device = 0;
	cudaStream_t stream = nullptr;
	gbfem_params prm{};
	int N = 0, E = 0, n = 0;
	int nb = 0, nl = 0;
	int64_t nnz = 0;
	bool active = true;
	int launches = 0;  // kernels launched by the current gbfem_step call
	std::string err;
	gbfem_stats stats{};

	// host structure
	std::vector<int32_t> tets;     // element node ids, npe() per element
	std::vector<int> adjPtr, adj;  // node adjacency incl. self (sorted) = BSR structure
	std::vector<double> cmass;     // per element rho V / 20 (consistent mass coefficient)
	std::vector<uint8_t> bcMask;
	std::vector<double> poissonHost;  // tetrahedra: per-element nu at creation (gbfem_set_materials_device)

	// device
	DevBuf<int4> d_tets;
	DevBuf<double> d_rest, d_xrest, d_lmass, d_nmass;
	DevBuf<int> d_perm, d_off, d_sellcol, d_cptr, d_cidx, d_iptr, d_iidx;
	int64_t sellSlots = 0;
	DevBuf<int4> d_lblk;
	DevBuf<uint8_t> d_bc;
	DevBuf<double> d_x, d_v, d_xt, d_vt;
	DevBuf<double> d_mu, d_adjG, d_gx, d_gv;  // differentiation form (allocated on first use)
	// Rollouts as CUDA graphs (gbfem_rollout_forward / _backward): checkpoints (the last slot holds the
	// final state), one segment's states, the adjoint pair (lx | lv), the gradients (log E | nu), the
	// step's velocity increment, and the adjoint solves' statistics.
	double rollDt = 0.0;
	int rollSteps = 0, rollEvery = 0, rollFwdVersion = -1, rollBwdVersion = -1;
	cudaGraphExec_t rollFwd = nullptr, rollBwd = nullptr;
	DevBuf<double> d_ckpt, d_segX, d_rollL, d_rollG, d_dvTmp, d_adjAcc;
	DevBuf<double> d_kslots, d_rhsE, d_A, d_invdiag, d_rhs, d_dv, d_dvPrev, d_r, d_p, d_q, d_part;
	// mixed-precision form
	DevBuf<float> d_rest32, d_kslots32, d_rhsE32, d_A32, d_invdiag32, d_xd, d_invd, d_r32, d_pA, d_pB, d_q32;
	DevBuf<double> d_brs, d_r64, d_x64;
	DevBuf<double> d_invd64, d_q64, d_zA64, d_zB64;  // FP64 batches: row-space vectors of the persistent solve
	DevBuf<int> d_rcol, d_segChunk, d_cumW;  // row-space columns, chunk range per segment, chunk weights
	DevBuf<double> d_slots;                  // cross-CTA partials of the persistent solve
	DevBuf<int> d_segMaxIter;                // default CG cap of each segment: 2 n_segment + 64
	int segMaxIterMax = 0;
	int maxChunksPerCta = 0;
	size_t pcgSmem = 0;
	// Tuning of the mixed form (picked by the autotuner or set by gbfem_set_tuning).
	int smCount = 0, chunkWeightMin = 1;
	int64_t chunkWeightTotal = 0;
	int ctasPerSM = 4, refreshWeight = kRefreshWeightDefault, elemsPerBlock = 64;
	int cgSchedule = kPcgMixed1;  // PcgForm of the mixed solve, set at creation from the system's size
	bool tuned = false;
	int tuneVersion = 0;
	// CUDA graph of one mixed-form step (GBFEM_STEP_GRAPH), rebuilt when dt, the timing flag or the
	// tuning changes.
	cudaGraphExec_t graphExec = nullptr;
	double graphDt = 0.0;
	bool graphTimed = false;
	int graphVersion = -1;
	DevBuf<double> d_acc;                    // per-segment statistics of graph-launched steps
	cudaEvent_t graphEv[2] = {nullptr, nullptr};
	DevBuf<SegCtl> d_seg;
	DevBuf<PcgGlobal> d_pcgGlobal;
	SegCtl* h_seg = nullptr;
	int pcgGrid = 0;
	// segments (meshes of a batch): node and tet ranges, chunk ranges
	std::vector<int> segNode{0}, segTet{0};
	std::vector<double> segStats;  // per segment over the last gbfem_step: iterations, refreshes, converged, residual
	int nrows = 0, nchunks = 0;
	bool mixed() const { return prm.precision == GBFEM_PRECISION_MIXED; }
	// A batch of meshes (segments); its solve is the persistent launch in either precision.
	bool batched() const { return segNode.size() > 2; }
	// Solved by the persistent launch (k_pcg_persistent): the mixed form, and FP64 batches.
	bool persistent() const { return mixed() || batched(); }
	bool linear() const { return prm.element_type == GBFEM_ELEMENT_LINEAR_TET; }
	bool hex() const { return prm.element_type == GBFEM_ELEMENT_HEXAHEDRON; }
	bool corotational() const { return prm.element_type == GBFEM_ELEMENT_COROTATIONAL_TET; }
	// CG iteration cap of a step: the caller's, else Eigen's default 2n. The mixed form's default adds
	// 64: FP32 CG loses conjugacy on very small systems and was measured needing up to ~2.5 n iterations
	// there (18-27 free dofs at tolerance 1e-12), where FP64 needs at most n; at scale the counts match.
	int stepMaxIter() const
	{
		return prm.cg_max_iterations > 0 ? prm.cg_max_iterations : (mixed() ? 2 * n + 64 : 2 * n);
	}
	int npe() const { return hex() ? 8 : 4; }
	// Constant system (linear elements): S is formed once per dt and materials.
	bool constantSystem() const { return !corotational(); }
	bool systemCurrent(double dt) const { return constantSystem() && linearReady && linearDt == dt; }
	// Hexahedra: element node ids, materials, and the assembled K / scalar block masses (SELL layout).
	DevBuf<int> d_enodes;
	DevBuf<double> d_young, d_poisson, d_rho, d_K, d_Ms, d_uw;
	DevBuf<float2> d_Kp, d_Msp;  // mixed form: K and the slot masses as float pairs (right-hand side)
	// Mixed form, corotational: per-element rest edges (FP32) and rest Gram (FP64).
	DevBuf<float> d_qf32;
	DevBuf<float2> d_qg2;
	// Node pass outputs of the FP32 corotational element kernel (x as float pairs, v, x - x_t, v - v_t).
	DevBuf<float2> d_nodeX;
	DevBuf<float> d_nodeV, d_nodeDx, d_nodeDv;
	int graphKernels = 0;  // kernels one launch of the captured step graph runs
	// External generalized forces for the next step (gbfem_add_external_force): node forces, and
	// K (9) and D (9) per node pair keyed I * N + J; the lower-block map to place them in S.
	bool extPending = false, extActive = false;
	std::vector<double> extF;
	std::map<int64_t, std::array<double, 18>> extBlocks;
	std::vector<int> lowerOfPosHost;
	std::vector<int4> lblkHost;
	DevBuf<unsigned char> d_ext;
	// Linear elements: the system matrix assembled for linearDt stays valid until dt or a material
	// changes (OdeSolverLinearEulerImplicit keeps its first step's system).
	bool linearReady = false;
	double linearDt = 0.0;
	// Compliance (gbfem_apply_compliance): the system matrix of the last step, and its dt.
	bool systemReady = false;
	double lastDt = 0.0;
	DevBuf<double> d_mcgVec, d_mcgPart, d_Re, d_Wn, d_xprev;
	DevBuf<McgCtl> d_mcgCtl;
	McgCtl* h_mcgCtl = nullptr;
	DevBuf<int> d_counters;
	DevBuf<CgCtl> d_ctl;
	CgCtl* h_ctl = nullptr;
	DevBuf<int> d_idx;      // scratch for gbfem_set_velocities
	DevBuf<double> d_vals;

	// export of the full system (allocated on first use)
	bool haveSystem = false;
	DevBuf<double> d_kfull, d_fE, d_S, d_smass, d_f;
	DevBuf<int> d_sptr, d_sidx, d_srow, d_scol;

	DevBody body() const
	{
		DevBody b;
		b.N = N;
		b.E = E;
		b.n = n;
		b.nb = nb;
		b.nl = nl;
		b.tets = d_tets.p;
		b.rest = d_rest.p;
		b.rest32 = d_rest32.p;
		b.xrest = d_xrest.p;
		b.lblk = d_lblk.p;
		b.cptr = d_cptr.p;
		b.cidx = d_cidx.p;
		b.lmass = d_lmass.p;
		b.iptr = d_iptr.p;
		b.iidx = d_iidx.p;
		b.nmass = d_nmass.p;
		b.bc = d_bc.p;
		b.qf32 = d_qf32.p;
		b.qg2 = d_qg2.p;
		b.nodeX = d_nodeX.p;
		b.nodeV = d_nodeV.p;
		b.nodeDx = d_nodeDx.p;
		b.nodeDv = d_nodeDv.p;
		b.lumped = prm.mass_lumping ? 1 : 0;
		return b;
	}

	Launch launch() const
	{
		Launch L;
		L.stream = stream;
		int g = (n + 255) / 256;
		L.vecGrid = std::max(1, std::min(g, 152 * 8));
		return L;
	}

	int blockPos(int I, int J) const
	{
		auto b = adj.begin() + adjPtr[I], e = adj.begin() + adjPtr[I + 1];
		auto it = std::lower_bound(b, e, J);
		return (it != e && *it == J) ? (int)(it - adj.begin()) : -1;
	}
	int64_t cscSlot(int r, int c) const
	{
		int I = r / 3, i = r % 3, J = c / 3, j = c % 3;
		int pos = blockPos(J, I);  // position of I in adj(J)
		if (pos < 0) return -1;
		int deg = adjPtr[J + 1] - adjPtr[J];
		return 9LL * adjPtr[J] + 3LL * j * deg + 3LL * (pos - adjPtr[J]) + i;
	}

	void release()
	{
		if (h_ctl) cudaFreeHost(h_ctl);
		h_ctl = nullptr;
		DevBuf<int4>* b4[] = {&d_tets, &d_lblk};
		for (auto* b : b4) b->free();
		if (h_seg) cudaFreeHost(h_seg);
		h_seg = nullptr;
		DevBuf<float>* bf[] = {&d_rest32, &d_kslots32, &d_rhsE32, &d_A32, &d_invdiag32, &d_xd, &d_invd, &d_r32,
							   &d_pA, &d_pB, &d_q32};
		for (auto* b : bf) b->free();
		for (auto* b : {&d_brs, &d_r64, &d_x64, &d_invd64, &d_q64, &d_zA64, &d_zB64}) b->free();
		for (auto* b : {&d_rcol, &d_segChunk, &d_cumW, &d_segMaxIter}) b->free();
		d_slots.free();
		d_acc.free();
		for (auto* b : {&d_mcgVec, &d_mcgPart, &d_Re, &d_Wn, &d_xprev}) b->free();
		d_mcgCtl.free();
		if (h_mcgCtl) cudaFreeHost(h_mcgCtl);
		h_mcgCtl = nullptr;
		if (graphExec) cudaGraphExecDestroy(graphExec);
		graphExec = nullptr;
		for (auto& e : graphEv)
			if (e) cudaEventDestroy(e);
		d_seg.free();
		d_pcgGlobal.free();
		for (auto* b : {&d_mu, &d_adjG, &d_gx, &d_gv, &d_ckpt, &d_segX, &d_rollL, &d_rollG, &d_dvTmp, &d_adjAcc}) b->free();
		if (rollFwd) cudaGraphExecDestroy(rollFwd);
		if (rollBwd) cudaGraphExecDestroy(rollBwd);
		rollFwd = rollBwd = nullptr;
		DevBuf<double>* bd[] = {&d_rest, &d_xrest, &d_lmass, &d_nmass, &d_x, &d_v, &d_xt, &d_vt, &d_kslots,
								&d_rhsE, &d_A, &d_invdiag, &d_rhs, &d_dv, &d_dvPrev, &d_r, &d_p, &d_q, &d_part,
								&d_vals, &d_kfull, &d_fE, &d_S, &d_smass, &d_f, &d_young, &d_poisson, &d_rho,
								&d_K, &d_Ms, &d_uw};
		for (auto* b : bd) b->free();
		d_Kp.free();
		d_Msp.free();
		DevBuf<int>* bi[] = {&d_perm, &d_off, &d_sellcol, &d_cptr, &d_cidx, &d_iptr, &d_iidx, &d_counters, &d_idx,
							 &d_sptr, &d_sidx, &d_srow, &d_scol, &d_enodes};
		for (auto* b : bi) b->free();
		d_ext.free();
		d_qf32.free();
		d_qg2.free();
		d_nodeX.free();
		for (auto* b : {&d_nodeV, &d_nodeDx, &d_nodeDv}) b->free();
		d_bc.free();
		d_ctl.free();
		if (stream) cudaStreamDestroy(stream);
		stream = nullptr;
	}
};

namespace gbfem {
// Message returned by gbfem_last_error(NULL, ...) (create failures, the no-allocation solve).
void set_global_error(const std::string& msg) { g_lastCreateError = msg; }
}  // namespace gbfem

namespace {

gbfem_status fail(gbfem_handle h, gbfem_status st, const std::string& msg)
{
	if (h)
		h->err = msg;
	else
		g_lastCreateError = msg;
	return st;
}

#define GB_CUDA(h, call)                                                                                 \
	do                                                                                                   \
	{                                                                                                    \
		cudaError_t e_ = (call);                                                                         \
		if (e_ != cudaSuccess)                                                                           \
			return fail(h, e_ == cudaErrorMemoryAllocation ? GBFEM_OUT_OF_MEMORY : GBFEM_CUDA_ERROR,     \
						std::string(#call) + ": " + cudaGetErrorString(e_));                            \
	} while (0)

// The persistent solve's dynamic shared memory limit is a process-wide attribute of the kernel:
// only ever raised, so a launch sized for one handle never breaks another's.
cudaError_t raise_pcg_smem_limit(size_t bytes, int form)
{
	static std::mutex mu;
	static size_t current[3] = {48 * 1024, 48 * 1024, 48 * 1024};
	std::lock_guard<std::mutex> lock(mu);
	if (bytes <= current[form]) return cudaSuccess;
	const cudaError_t e = pcg_set_max_dynamic_smem(form, (int)bytes);
	if (e == cudaSuccess) current[form] = bytes;
	return e;
}

// Grid of the persistent solve for `cps` CTAs per SM and the handle's refresh weight rw:
// G = min(cps * SMs, chunks); the largest share of a CTA in chunks (its shared-memory partials) is
// bounded from the chunk weights: a weighted share holds fewer than tot / (G wmin) + 1 chunks (tot at
// most rw times the plain total, a refreshing segment's chunks weighing rw times theirs), a counted one
// at most ceil(n / G). Fails if that many CTAs do not fit on an SM. Called again whenever rw changes.
gbfem_status configure_pcg(gbfem_handle h, int cps)
{
	const int nseg = (int)h->segNode.size() - 1;
	const int G = std::max(1, std::min(cps * h->smCount, h->nchunks));
	const int64_t rw = std::max(1, h->refreshWeight);
	const int64_t mW = rw * h->chunkWeightTotal / ((int64_t)G * h->chunkWeightMin) + 2;
	const int64_t mC = (int64_t)h->nchunks / G + 2;
	const int M = (int)std::max(mW, mC);
	const size_t smem = pcg_smem_bytes(nseg, M);
	if (smem > 160 * 1024) return fail(h, GBFEM_INVALID_ARG, "batch too large for the persistent solve");
	const int form = h->mixed() ? h->cgSchedule : kPcgF64;
	GB_CUDA(h, raise_pcg_smem_limit(smem, form));
	int perSM = 0;
	GB_CUDA(h, pcg_occupancy(form, &perSM, smem));
	if (perSM < std::min(cps, (G + h->smCount - 1) / h->smCount))
		return fail(h, GBFEM_INVALID_ARG, "persistent solve: " + std::to_string(cps) + " CTAs per SM do not fit");
	h->pcgGrid = G;
	h->maxChunksPerCta = M;
	h->pcgSmem = smem;
	h->ctasPerSM = cps;
	return GBFEM_OK;
}

// Hexahedra: element integrals from the current materials, assembled into K and the scalar block
// masses (also the per-lower-block masses S is formed from). Any stored system is then stale.
gbfem_status rebuild_hex_operators(gbfem_handle h)
{
	cudaStream_t s = h->stream;
	struct Scratch
	{
		DevBuf<double> slots, smass, rowsum;
		~Scratch()
		{
			slots.free();
			smass.free();
			rowsum.free();
		}
	} t;
	GB_CUDA(h, t.slots.alloc((size_t)h->E * kHexSlots * 9));
	GB_CUDA(h, t.smass.alloc((size_t)h->E * kHexSlots));
	launch_hex_element(h->E, h->d_enodes.p, h->d_xrest.p, h->d_young.p, h->d_poisson.p, h->d_rho.p, t.slots.p,
					   t.smass.p, s);
	launch_assemble_k(h->body(), t.slots.p, t.smass.p, h->d_K.p, h->d_Ms.p, h->d_lmass.p, s);
	if (h->prm.mass_lumping)
	{
		GB_CUDA(h, t.rowsum.alloc((size_t)h->N));
		const MatSell3 K{h->nrows, h->d_perm.p, h->d_off.p, h->d_sellcol.p, h->d_K.p};
		launch_hex_lump_masses(h->body(), K, h->d_Ms.p, h->d_lmass.p, t.rowsum.p, s);
	}
	if (h->mixed())
	{
		const size_t slots = (size_t)h->sellSlots;
		if (!h->d_Kp.p) GB_CUDA(h, h->d_Kp.alloc(9 * slots));
		if (!h->d_Msp.p) GB_CUDA(h, h->d_Msp.alloc(slots));
		launch_split_pairs(9 * slots, h->d_K.p, h->d_Kp.p, s);
		launch_split_pairs(slots, h->d_Ms.p, h->d_Msp.p, s);
	}
	GB_CUDA(h, cudaGetLastError());
	GB_CUDA(h, cudaStreamSynchronize(s));  // before the scratch is released
	h->linearReady = false;
	return GBFEM_OK;
}

// Everything the step needs from the mesh, computed on the host once.
gbfem_status build_body(gbfem_handle h, const gbfem_mesh_desc* m)
{
	const int N = m->num_nodes, E = m->num_tets;
	if (!h->hex()) h->poissonHost.assign(m->poisson_ratio, m->poisson_ratio + E);
	h->N = N;
	h->E = E;
	h->n = 3 * N;
	const int npe = h->npe();
	h->tets.assign(m->tets, m->tets + npe * (size_t)E);
	const double* X = m->rest_positions;

	// Rest precompute (Fem3DElementTetrahedron.cpp:92-216; Fem3DElementCorotationalTetrahedron.cpp:57-72).
	std::vector<double> rest(h->hex() ? 0 : (size_t)kRestFields * E);
	h->cmass.resize(h->hex() ? 0 : E);
	std::vector<double> elemMass(E);
	for (int e = 0; e < E && h->hex(); ++e)
	{
		double vol = 0.0;
		hex_rest_check(X, &h->tets[8 * (size_t)e], &vol);  // validated before
		elemMass[e] = vol * m->mass_density[e];            // FemElement::getMass
	}
	for (int e = 0; e < E && !h->hex(); ++e)
	{
		const int* nd = &h->tets[4 * (size_t)e];
		for (int a = 0; a < 4; ++a)
			for (int b = a + 1; b < 4; ++b)
				if (nd[a] == nd[b]) return fail(h, GBFEM_INVALID_ARG, "tet " + std::to_string(e) + " repeats a node");
		double V[4][4], Vi[4][4];
		for (int a = 0; a < 4; ++a)
		{
			for (int k = 0; k < 3; ++k) V[k][a] = X[3 * (size_t)nd[a] + k];
			V[3][a] = 1.0;
		}
		if (!inverse44(V, Vi))
			return fail(h, GBFEM_DEGENERATE_ELEMENT,
						"tet " + std::to_string(e) + ": matrix V not invertible (degenerated tetrahedron)");
		const double* p0 = X + 3 * (size_t)nd[0];
		const double* p1 = X + 3 * (size_t)nd[1];
		const double* p2 = X + 3 * (size_t)nd[2];
		const double* p3 = X + 3 * (size_t)nd[3];
		const double vol = (det3v(p1, p2, p3) - det3v(p0, p2, p3) + det3v(p0, p1, p3) - det3v(p0, p1, p2)) / 6.0;
		const double Ey = m->young_modulus[e], nu = m->poisson_ratio[e], rho = m->mass_density[e];
		const double lambda = Ey * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
		const double mu = Ey / (2.0 * (1 + nu));
		for (int a = 0; a < 4; ++a)
			for (int k = 0; k < 3; ++k) rest[(size_t)(3 * a + k) * E + e] = Vi[a][k];
		rest[(size_t)12 * E + e] = vol;
		rest[(size_t)13 * E + e] = lambda * vol;
		rest[(size_t)14 * E + e] = mu * vol;
		rest[(size_t)15 * E + e] = vol * rho / 20.0;
		h->cmass[e] = vol * rho / 20.0;
		elemMass[e] = vol * rho;  // FemElement::getMass
	}
	// Node adjacency (the union of element node blocks, FemRepresentation.cpp:121-132).
	std::vector<int> cnt(N + 1, 0);
	for (int e = 0; e < E; ++e)
		for (int a = 0; a < npe; ++a) cnt[h->tets[npe * (size_t)e + a] + 1] += npe;
	for (int i = 0; i < N; ++i) cnt[i + 1] += cnt[i];
	std::vector<int> raw(cnt[N]);
	{
		std::vector<int> fill(cnt.begin(), cnt.end() - 1);
		for (int e = 0; e < E; ++e)
			for (int a = 0; a < npe; ++a)
				for (int b = 0; b < npe; ++b)
					raw[fill[h->tets[npe * (size_t)e + a]]++] = h->tets[npe * (size_t)e + b];
	}
	h->adjPtr.assign(N + 1, 0);
	h->adj.clear();
	h->adj.reserve(raw.size() / 3 + N);
	for (int i = 0; i < N; ++i)
	{
		auto b = raw.begin() + cnt[i], en = raw.begin() + cnt[i + 1];
		std::sort(b, en);
		auto last = std::unique(b, en);
		if (b == last) h->adj.push_back(i);  // isolated node: keep its diagonal block
		else h->adj.insert(h->adj.end(), b, last);
		h->adjPtr[i + 1] = (int)h->adj.size();
	}
	h->nb = (int)h->adj.size();
	h->nnz = 9LL * h->nb;
	if (h->nnz > INT32_MAX) return fail(h, GBFEM_INVALID_ARG, "pattern exceeds int32 indices");
	// SELL-32 layout of the block matrix. Inside each segment (mesh of a batch) rows are sorted by
	// block count (descending, stable); each segment is padded to a multiple of 32 rows so that a
	// chunk of 32 rows never straddles two segments. perm[row] = node id, -1 on padding rows.
	const int nseg = (int)h->segNode.size() - 1;
	std::vector<int> perm, chunkSeg, segChunk(nseg + 1, 0);
	for (int sg = 0; sg < nseg; ++sg)
	{
		const int n0 = h->segNode[sg], n1 = h->segNode[sg + 1];
		std::vector<int> rows(n1 - n0);
		for (int i = n0; i < n1; ++i) rows[i - n0] = i;
		std::stable_sort(rows.begin(), rows.end(), [&](int a, int b) {
			return (h->adjPtr[a + 1] - h->adjPtr[a]) > (h->adjPtr[b + 1] - h->adjPtr[b]);
		});
		rows.resize((rows.size() + 31) / 32 * 32, -1);
		perm.insert(perm.end(), rows.begin(), rows.end());
		for (size_t c = 0; c < rows.size() / 32; ++c) chunkSeg.push_back(sg);
		segChunk[sg + 1] = (int)chunkSeg.size();
	}
	const int nrows = (int)perm.size();
	const int nchunks = nrows / 32;
	std::vector<int> off(nchunks + 1, 0), iperm(N, -1), sellBase(h->nb);
	for (int rs = 0; rs < nrows; ++rs)
		if (perm[rs] >= 0) iperm[perm[rs]] = rs;
	for (int c = 0; c < nchunks; ++c)
	{
		int w = 0;
		for (int l = 0; l < 32; ++l)
		{
			const int I = perm[32 * c + l];
			if (I >= 0) w = std::max(w, h->adjPtr[I + 1] - h->adjPtr[I]);
		}
		off[c + 1] = off[c] + w;
	}
	const int64_t sellSlots = 32LL * off[nchunks];
	if (sellSlots * 9 > INT32_MAX) return fail(h, GBFEM_INVALID_ARG, "matrix exceeds int32 indices");
	// Column of each slot as a node id (FP64 form, dof-space vectors) and as a row position (mixed
	// form, row-space vectors). Padding slots point at the row itself with zero values.
	std::vector<int> scol(sellSlots, 0), rcol(sellSlots, 0);
	for (int rs = 0; rs < nrows; ++rs)
	{
		const int I = perm[rs], c = rs >> 5, lane = rs & 31;
		const int deg = (I >= 0) ? h->adjPtr[I + 1] - h->adjPtr[I] : 0;
		for (int t = 0; t < off[c + 1] - off[c]; ++t)
		{
			const int k = off[c] + t;
			const int J = (t < deg) ? h->adj[h->adjPtr[I] + t] : (I >= 0 ? I : perm[32 * c]);
			scol[(size_t)k * 32 + lane] = J;
			rcol[(size_t)k * 32 + lane] = (t < deg) ? iperm[J] : rs;
			if (t < deg) sellBase[h->adjPtr[I] + t] = k * 288 + lane;
		}
	}
	for (int64_t k = 0; k < sellSlots; ++k)  // host-side bounds check of every index the kernels follow
		if (scol[k] < 0 || scol[k] >= N || rcol[k] < 0 || rcol[k] >= nrows)
			return fail(h, GBFEM_CUDA_ERROR, "internal error: SELL index out of range");
	h->sellSlots = sellSlots;
	h->nrows = nrows;
	h->nchunks = nchunks;
	// Lower blocks (I >= J), collected in row order, each written to the SELL positions of (I,J) and (J,I).
	std::vector<int> lowerOfPos(h->nb, -1);
	std::vector<int4> lblk;
	lblk.reserve(h->nb / 2 + N);
	for (int I = 0; I < N; ++I)
		for (int k = h->adjPtr[I]; k < h->adjPtr[I + 1]; ++k)
		{
			int J = h->adj[k];
			if (J > I) continue;
			lowerOfPos[k] = (int)lblk.size();
			lblk.push_back(make_int4(I, J, sellBase[k], I == J ? -1 : sellBase[h->blockPos(J, I)]));
		}
	// Assembly threads run in the order of the (I,J) blocks' SELL positions, so the lanes of a warp
	// write neighbouring lanes of one SELL block column (coalesced) instead of one row's blocks, whose
	// positions are 288 values apart. Each block's sum is unchanged (its contributions stay in element
	// order); only which thread forms it moves.
	{
		std::vector<int> order(lblk.size());
		for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
		std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return lblk[x].z < lblk[y].z; });
		std::vector<int> newIndex(lblk.size());
		std::vector<int4> sorted(lblk.size());
		for (size_t i = 0; i < order.size(); ++i)
		{
			newIndex[order[i]] = (int)i;
			sorted[i] = lblk[order[i]];
		}
		lblk.swap(sorted);
		for (int& L : lowerOfPos)
			if (L >= 0) L = newIndex[L];
	}
	h->nl = (int)lblk.size();
	h->lowerOfPosHost = lowerOfPos;
	h->lblkHost = lblk;
	// Element slot -> lower block contributions, element order inside each block. Slots: the npe
	// diagonal blocks, then the node pairs a < b in lexicographic order.
	const int spe = h->hex() ? kHexSlots : kSlots;
	std::vector<int> pa, pb;
	for (int a = 0; a < npe; ++a)
	{
		pa.push_back(a);
		pb.push_back(a);
	}
	for (int a = 0; a < npe; ++a)
		for (int b = a + 1; b < npe; ++b)
		{
			pa.push_back(a);
			pb.push_back(b);
		}
	std::vector<int> slotLower((size_t)E * spe);
	std::vector<int> cptr(h->nl + 1, 0);
	for (int e = 0; e < E; ++e)
	{
		const int* nd = &h->tets[npe * (size_t)e];
		for (int s = 0; s < spe; ++s)
		{
			const int I = std::max(nd[pa[s]], nd[pb[s]]), J = std::min(nd[pa[s]], nd[pb[s]]);
			int L = lowerOfPos[h->blockPos(I, J)];
			slotLower[(size_t)e * spe + s] = L;
			cptr[L + 1]++;
		}
	}
	for (int L = 0; L < h->nl; ++L) cptr[L + 1] += cptr[L];
	std::vector<int> cidx((size_t)E * spe);
	std::vector<double> lmass(h->nl, 0.0);  // hexahedra: summed on the device from the element integrals
	{
		std::vector<int> fill(cptr.begin(), cptr.end() - 1);
		for (int e = 0; e < E; ++e)
			for (int s = 0; s < spe; ++s)
			{
				int L = slotLower[(size_t)e * spe + s];
				cidx[fill[L]++] = e * spe + s;
				// Consistent mass rho V / 20 ([2 on the diagonal, 1 off] x I3); with mass lumping each row
				// summed onto the diagonal block: 5 cm = rho V / 4, off-diagonal blocks 0.
				if (!h->hex())
					lmass[L] += h->prm.mass_lumping ? (s < 4 ? 5.0 * h->cmass[e] : 0.0)
													: h->cmass[e] * (s < 4 ? 2.0 : 1.0);
			}
	}
	// Node incidences and lumped node masses getMass / numNodes (FemRepresentation.cpp:102-117).
	std::vector<int> iptr(N + 1, 0), iidx(npe * (size_t)E);
	for (int e = 0; e < E; ++e)
		for (int a = 0; a < npe; ++a) iptr[h->tets[npe * (size_t)e + a] + 1]++;
	for (int i = 0; i < N; ++i) iptr[i + 1] += iptr[i];
	std::vector<double> nmass(N, 0.0);
	{
		std::vector<int> fill(iptr.begin(), iptr.end() - 1);
		for (int e = 0; e < E; ++e)
			for (int a = 0; a < npe; ++a)
			{
				int I = h->tets[npe * (size_t)e + a];
				iidx[fill[I]++] = npe * e + a;
				nmass[I] += elemMass[e] / npe;
			}
	}
	h->bcMask.assign(h->n, 0);
	for (int i = 0; i < m->num_bc_dofs; ++i) h->bcMask[m->bc_dofs[i]] = 1;

	cudaStream_t s = h->stream;
	if (!h->hex())
	{
		GB_CUDA(h, h->d_tets.upload(reinterpret_cast<const int4*>(h->tets.data()), E, s));
		GB_CUDA(h, h->d_rest.upload(rest.data(), rest.size(), s));
	}
	GB_CUDA(h, h->d_xrest.upload(X, h->n, s));
	GB_CUDA(h, h->d_perm.upload(perm.data(), perm.size(), s));
	GB_CUDA(h, h->d_off.upload(off.data(), off.size(), s));
	GB_CUDA(h, h->d_sellcol.upload(scol.data(), scol.size(), s));
	if (h->persistent())
	{
		GB_CUDA(h, h->d_rcol.upload(rcol.data(), rcol.size(), s));
		GB_CUDA(h, h->d_segChunk.upload(segChunk.data(), segChunk.size(), s));
	}
	GB_CUDA(h, h->d_lblk.upload(lblk.data(), lblk.size(), s));
	GB_CUDA(h, h->d_cptr.upload(cptr.data(), cptr.size(), s));
	GB_CUDA(h, h->d_cidx.upload(cidx.data(), cidx.size(), s));
	GB_CUDA(h, h->d_lmass.upload(lmass.data(), lmass.size(), s));
	if (!h->hex())
	{
		GB_CUDA(h, h->d_iptr.upload(iptr.data(), iptr.size(), s));
		GB_CUDA(h, h->d_iidx.upload(iidx.data(), iidx.size(), s));
	}
	GB_CUDA(h, h->d_nmass.upload(nmass.data(), nmass.size(), s));
	GB_CUDA(h, h->d_bc.upload(h->bcMask.data(), h->bcMask.size(), s));
	GB_CUDA(h, h->d_x.upload(X, h->n, s));
	GB_CUDA(h, h->d_v.alloc(h->n));
	GB_CUDA(h, cudaMemsetAsync(h->d_v.p, 0, sizeof(double) * h->n, s));
	const size_t nv = h->n;
	if (h->hex())
	{
		// Element integrals once, assembled into K and the scalar block masses; the per-element
		// slots are released afterwards.
		GB_CUDA(h, h->d_enodes.upload(h->tets.data(), h->tets.size(), s));
		GB_CUDA(h, h->d_young.upload(m->young_modulus, E, s));
		GB_CUDA(h, h->d_poisson.upload(m->poisson_ratio, E, s));
		GB_CUDA(h, h->d_rho.upload(m->mass_density, E, s));
		GB_CUDA(h, h->d_K.alloc((size_t)sellSlots * 9));
		GB_CUDA(h, cudaMemsetAsync(h->d_K.p, 0, sizeof(double) * sellSlots * 9, s));  // padding blocks stay 0
		GB_CUDA(h, h->d_Ms.alloc((size_t)sellSlots));
		GB_CUDA(h, cudaMemsetAsync(h->d_Ms.p, 0, sizeof(double) * sellSlots, s));
		GB_CUDA(h, h->d_uw.alloc(6 * (size_t)N));
		gbfem_status st = rebuild_hex_operators(h);
		if (st != GBFEM_OK) return st;
	}
	// The persistent solve's control structures (mixed form, FP64 batches): per-segment CG state, the
	// chunk weights its partition balances, the grid and the per-segment iteration caps.
	auto setup_persistent = [&]() -> gbfem_status {
		GB_CUDA(h, h->d_seg.alloc(nseg));
		GB_CUDA(h, h->d_pcgGlobal.alloc(1));
		GB_CUDA(h, cudaMallocHost(&h->h_seg, sizeof(SegCtl) * nseg));
		// Persistent grid: as many co-resident CTAs as fit, at most 4 per SM. The kernel splits the
		// chunks of the segments still iterating over the CTAs itself; the host bounds the largest
		// share (shared-memory partials) from the chunk weights.
		std::vector<int> cumW(nchunks + 1, 0);
		int wmin = INT32_MAX;
		for (int c = 0; c < nchunks; ++c)
		{
			const int w = off[c + 1] - off[c] + kPcgChunkWeight;
			wmin = std::min(wmin, w);
			if ((int64_t)cumW[c] + w > INT32_MAX) return fail(h, GBFEM_INVALID_ARG, "matrix too large for the persistent solve");
			cumW[c + 1] = cumW[c] + w;
		}
		GB_CUDA(h, cudaDeviceGetAttribute(&h->smCount, cudaDevAttrMultiProcessorCount, h->device));
		h->chunkWeightTotal = cumW[nchunks];
		h->chunkWeightMin = std::max(1, wmin);
		// CG schedule until the autotuner or gbfem_set_tuning picks one: one grid phase an iteration
		// where a phase leaves each warp a few chunks (its phases wait on latency; one 1.28M-tet mesh,
		// 8,458 chunks: 17.2 vs 22.9 ms a solve), two phases where phases stream many chunks a warp
		// (64 meshes, 19,549 chunks: 15.7 vs 16.3 ms; 256 meshes: 41.3 vs 53.1 ms).
		h->cgSchedule = (nchunks <= kOnePhaseChunksPerSlot * 4 * h->smCount) ? kPcgMixed1 : kPcgMixed2;
		gbfem_status cst = GBFEM_INVALID_ARG;
		std::string why;
		for (int cps = 4; cps >= 1 && cst != GBFEM_OK; --cps)
		{
			cst = configure_pcg(h, cps);
			if (cst != GBFEM_OK) why += (why.empty() ? "" : "; ") + h->err;
		}
		if (cst != GBFEM_OK) return fail(h, cst, "persistent solve: no grid fits (" + why + ")");
		GB_CUDA(h, h->d_cumW.upload(cumW.data(), cumW.size(), s));
		GB_CUDA(h, h->d_slots.alloc(2 * kPcgNV * 4 * (size_t)h->smCount));  // any grid of up to 4 CTAs per SM
		// Each mesh of a batch has its own default CG cap, as each representation's solver would
		// (Eigen's 2n for its own n; the FP32 CG needs the extra 64 on systems of a few dozen dofs).
		std::vector<int> segCap(nseg);
		h->segMaxIterMax = 0;
		for (int sg = 0; sg < nseg; ++sg)
		{
			segCap[sg] = 2 * 3 * (h->segNode[sg + 1] - h->segNode[sg]) + (h->mixed() ? 64 : 0);
			h->segMaxIterMax = std::max(h->segMaxIterMax, segCap[sg]);
		}
		GB_CUDA(h, h->d_segMaxIter.upload(segCap.data(), segCap.size(), s));
		GB_CUDA(h, h->d_acc.alloc(4 * (size_t)nseg + 2));
		return GBFEM_OK;
	};
	if (!h->mixed())
	{
		if (!h->hex())
		{
			GB_CUDA(h, h->d_kslots.alloc((size_t)E * kSlots * 9));
			GB_CUDA(h, h->d_rhsE.alloc((size_t)E * 12));
		}
		GB_CUDA(h, h->d_A.alloc((size_t)sellSlots * 9));
		GB_CUDA(h, cudaMemsetAsync(h->d_A.p, 0, sizeof(double) * sellSlots * 9, s));  // padding blocks stay 0
		for (DevBuf<double>* b : {&h->d_invdiag, &h->d_r, &h->d_p, &h->d_q}) GB_CUDA(h, b->alloc(nv));
		if (h->batched())
		{
			// FP64 batch: the persistent FP64 CG's row-space vectors; z and p of a row in one 64-byte record.
			const size_t nr = 3 * (size_t)nrows;
			for (DevBuf<double>* b : {&h->d_invd64, &h->d_q64, &h->d_r64, &h->d_x64}) GB_CUDA(h, b->alloc(nr));
			for (DevBuf<double>* b : {&h->d_zA64, &h->d_zB64}) GB_CUDA(h, b->alloc(8 * (size_t)nrows));
			gbfem_status pst = setup_persistent();
			if (pst != GBFEM_OK) return pst;
			GB_CUDA(h, cudaStreamSynchronize(s));
		}
	}
	else
	{
		if (h->corotational())
		{
			// Rest edges q_a = x0_a - x0_0 (FP32) and their Gram q_a . q_c (an unevaluated float pair:
			// hi = the FP64 Gram rounded, lo = the rest rounded) per element, so the FP32 element kernel
			// neither gathers rest positions nor recomputes these constants each step.
			std::vector<float> qf((size_t)9 * E);
			std::vector<float2> qg((size_t)6 * E);
			for (int e = 0; e < E; ++e)
			{
				const int32_t* nd = &h->tets[4 * (size_t)e];
				double q[4][3];
				for (int a = 0; a < 4; ++a)
					for (int k = 0; k < 3; ++k) q[a][k] = X[3 * (size_t)nd[a] + k] - X[3 * (size_t)nd[0] + k];
				for (int a = 1; a < 4; ++a)
					for (int k = 0; k < 3; ++k) qf[(size_t)(3 * (a - 1) + k) * E + e] = float(q[a][k]);
				int pi = 0;
				for (int a = 1; a < 4; ++a)
					for (int c = a; c < 4; ++c)
					{
						const double gq = q[a][0] * q[c][0] + q[a][1] * q[c][1] + q[a][2] * q[c][2];
						const float hi = float(gq);
						qg[(size_t)(pi++) * E + e] = make_float2(hi, float(gq - double(hi)));
					}
			}
			GB_CUDA(h, h->d_qf32.upload(qf.data(), qf.size(), s));
			GB_CUDA(h, h->d_qg2.upload(qg.data(), qg.size(), s));
			GB_CUDA(h, h->d_nodeX.alloc(nv));
			for (DevBuf<float>* b : {&h->d_nodeV, &h->d_nodeDx, &h->d_nodeDv}) GB_CUDA(h, b->alloc(nv));
			GB_CUDA(h, cudaStreamSynchronize(s));
		}
		if (!h->hex())
		{
			// FP32 copy of the FP64 rest precompute (K0 and volume stay FP64-derived).
			std::vector<float> rest32(rest.begin(), rest.end());
			GB_CUDA(h, h->d_rest32.upload(rest32.data(), rest32.size(), s));
			GB_CUDA(h, cudaStreamSynchronize(s));
			GB_CUDA(h, h->d_kslots32.alloc((size_t)E * kSlots * 9));
			GB_CUDA(h, h->d_rhsE32.alloc((size_t)E * 12));
		}
		GB_CUDA(h, h->d_A32.alloc((size_t)sellSlots * 9));
		GB_CUDA(h, cudaMemsetAsync(h->d_A32.p, 0, sizeof(float) * sellSlots * 9, s));
		GB_CUDA(h, h->d_invdiag32.alloc(nv));
		const size_t nr = 3 * (size_t)nrows;  // row-space vectors of the persistent solve
		for (DevBuf<float>* b : {&h->d_xd, &h->d_invd, &h->d_r32, &h->d_q32}) GB_CUDA(h, b->alloc(nr));
		// The rows' records that neighbours gather: two-phase schedule, z and p in 32 bytes (one sector);
		// one-phase schedule, {r, w, s} and invdiag in 48 bytes.
		for (DevBuf<float>* b : {&h->d_pA, &h->d_pB}) GB_CUDA(h, b->alloc(12 * (size_t)nrows));
		for (DevBuf<double>* b : {&h->d_brs, &h->d_r64, &h->d_x64}) GB_CUDA(h, b->alloc(nr));
		gbfem_status pst = setup_persistent();
		if (pst != GBFEM_OK) return pst;
		GB_CUDA(h, cudaStreamSynchronize(s));
	}
	for (DevBuf<double>* b : {&h->d_rhs, &h->d_dv}) GB_CUDA(h, b->alloc(nv));
	GB_CUDA(h, h->d_part.alloc(partial_slots(h->launch().vecGrid)));
	GB_CUDA(h, h->d_counters.alloc(4));
	GB_CUDA(h, cudaMemsetAsync(h->d_counters.p, 0, 4 * sizeof(int), s));
	GB_CUDA(h, h->d_ctl.alloc(1));
	GB_CUDA(h, cudaMemsetAsync(h->d_ctl.p, 0, sizeof(CgCtl), s));
	GB_CUDA(h, cudaMallocHost(&h->h_ctl, sizeof(CgCtl)));
	GB_CUDA(h, cudaStreamSynchronize(s));
	return GBFEM_OK;
}

// Lazily built maps for exporting the full (non-mirrored) system in CSC order.
gbfem_status ensure_system_maps(gbfem_handle h)
{
	if (h->d_sptr.p) return GBFEM_OK;
	const int E = h->E;
	const int64_t nnz = h->nnz;
	std::vector<int> slot((size_t)E * 144);
	std::vector<int> sptr(nnz + 1, 0);
	for (int e = 0; e < E; ++e)
	{
		const int* nd = &h->tets[4 * (size_t)e];
		for (int a = 0; a < 4; ++a)
			for (int i = 0; i < 3; ++i)
				for (int b = 0; b < 4; ++b)
					for (int j = 0; j < 3; ++j)
					{
						int64_t k = h->cscSlot(3 * nd[a] + i, 3 * nd[b] + j);
						slot[(size_t)e * 144 + (3 * a + i) * 12 + 3 * b + j] = (int)k;
						sptr[k + 1]++;
					}
	}
	for (int64_t k = 0; k < nnz; ++k) sptr[k + 1] += sptr[k];
	std::vector<int> sidx((size_t)E * 144), srow(nnz), scol(nnz);
	std::vector<double> smass(nnz, 0.0);
	std::vector<int> fill(sptr.begin(), sptr.end() - 1);
	for (int e = 0; e < E; ++e)
		for (int l = 0; l < 144; ++l)
		{
			int k = slot[(size_t)e * 144 + l];
			sidx[fill[k]++] = e * 144 + l;
			int a = l / 36, i = (l / 12) % 3, b = (l % 12) / 3, j = l % 3;
			if (i == j)
				smass[k] += h->prm.mass_lumping ? (a == b ? 5.0 * h->cmass[e] : 0.0) : h->cmass[e] * (a == b ? 2.0 : 1.0);
		}
	for (int J = 0; J < h->N; ++J)
		for (int j = 0; j < 3; ++j)
		{
			int c = 3 * J + j;
			int deg = h->adjPtr[J + 1] - h->adjPtr[J];
			int64_t k = 9LL * h->adjPtr[J] + 3LL * j * deg;
			for (int t = h->adjPtr[J]; t < h->adjPtr[J + 1]; ++t)
				for (int i = 0; i < 3; ++i, ++k)
				{
					srow[k] = 3 * h->adj[t] + i;
					scol[k] = c;
				}
		}
	cudaStream_t s = h->stream;
	GB_CUDA(h, h->d_sptr.upload(sptr.data(), sptr.size(), s));
	GB_CUDA(h, h->d_sidx.upload(sidx.data(), sidx.size(), s));
	GB_CUDA(h, h->d_srow.upload(srow.data(), srow.size(), s));
	GB_CUDA(h, h->d_scol.upload(scol.data(), scol.size(), s));
	GB_CUDA(h, h->d_smass.upload(smass.data(), smass.size(), s));
	GB_CUDA(h, h->d_kfull.alloc((size_t)E * 144));
	GB_CUDA(h, h->d_fE.alloc((size_t)E * 12));
	GB_CUDA(h, h->d_S.alloc(nnz));
	GB_CUDA(h, h->d_f.alloc(h->n));
	GB_CUDA(h, cudaStreamSynchronize(s));
	return GBFEM_OK;
}

struct PhaseTimer
{
	bool on = false;
	cudaStream_t s = nullptr;
	cudaEvent_t ev[5] = {};
	void init(bool enable, cudaStream_t st)
	{
		on = enable;
		s = st;
		if (on)
			for (auto& e : ev) cudaEventCreate(&e);
	}
	void mark(int i)
	{
		if (on) cudaEventRecord(ev[i], s);
	}
	float ms(int a, int b)
	{
		float t = 0;
		if (on) cudaEventElapsedTime(&t, ev[a], ev[b]);
		return t;
	}
	~PhaseTimer()
	{
		if (on)
			for (auto& e : ev) cudaEventDestroy(e);
	}
};

// CUDA events bracketing individual kernel launches (GBFEM_STEP_TIME_KERNELS).
struct KernelTimer
{
	static constexpr int kPairs = 32;
	cudaEvent_t a[kPairs] = {}, b[kPairs] = {};
	bool ready = false;
	bool init()
	{
		if (ready) return true;
		for (int i = 0; i < kPairs; ++i)
			if (cudaEventCreate(&a[i]) != cudaSuccess || cudaEventCreate(&b[i]) != cudaSuccess) return false;
		ready = true;
		return true;
	}
	~KernelTimer()
	{
		if (ready)
			for (int i = 0; i < kPairs; ++i)
			{
				cudaEventDestroy(a[i]);
				cudaEventDestroy(b[i]);
			}
	}
};

// Jacobi PCG on the handle's symmetric BSR matrix; the host polls the device control block
// between chunks of iterations (kernels after convergence return immediately).
gbfem_status run_cg(gbfem_handle h, const double* b, double* x, int maxIter, bool timeSpmv)
{
	static thread_local KernelTimer kt;
	if (timeSpmv && !kt.init()) return fail(h, GBFEM_CUDA_ERROR, "cudaEventCreate failed");
	const Launch L = h->launch();
	MatSell3 A{h->nrows, h->d_perm.p, h->d_off.p, h->d_sellcol.p, h->d_A.p};
	launch_cg_init(h->n, b, h->d_invdiag.p, x, h->d_r.p, h->d_p.p, h->d_ctl.p, h->d_part.p, h->prm.cg_tolerance,
				   maxIter, L);
	h->launches++;
	long long launched = 0;
	int chunk = 4;
	int iterBefore = 0;
	for (;;)
	{
		for (int k = 0; k < chunk; ++k)
		{
			if (timeSpmv) cudaEventRecord(kt.a[k], h->stream);
			launch_cg_spmv_sell(A, h->d_p.p, h->d_q.p, h->d_ctl.p, h->d_part.p, L);
			if (timeSpmv) cudaEventRecord(kt.b[k], h->stream);
			launch_cg_update(h->n, h->d_invdiag.p, h->d_p.p, h->d_q.p, x, h->d_r.p, h->d_ctl.p, h->d_part.p, L);
			launch_cg_pupdate(h->n, h->d_invdiag.p, h->d_r.p, h->d_p.p, h->d_ctl.p, L);
		}
		h->launches += 3 * chunk;
		launched += chunk;
		GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl.p, sizeof(CgCtl), cudaMemcpyDeviceToHost, h->stream));
		GB_CUDA(h, cudaStreamSynchronize(h->stream));
		if (timeSpmv)
		{
			// Launches that did work: one per iteration, plus the converging one.
			const CgCtl& c = *h->h_ctl;
			int real = c.iter - iterBefore + ((c.done && c.converged && c.bb > 0 && c.iter < c.maxIter) ? 1 : 0);
			real = std::max(0, std::min(real, chunk));
			for (int k = 0; k < real; ++k)
			{
				float ms = 0;
				cudaEventElapsedTime(&ms, kt.a[k], kt.b[k]);
				h->stats.ms_spmv += ms;
				h->stats.spmv_timed++;
			}
			iterBefore = c.iter;
		}
		if (h->h_ctl->done) break;
		if (launched > (long long)maxIter + 64) return fail(h, GBFEM_CUDA_ERROR, "CG control block did not finish");
		chunk = std::min(chunk * 2, KernelTimer::kPairs);
	}
	return GBFEM_OK;
}

// Mixed-precision solve: FP32 CG iterations with reliable FP64 residual refreshes; the host polls
// the device control block between chunks of iterations.
// Enqueue one persistent solve on the handle's stream (no host synchronisation; capturable).
// ev0/ev1 (optional) bracket the solve; inside a stream capture they are recorded as external event
// nodes (a plain record there would only become a dependency edge and never record the event).
gbfem_status enqueue_mixed(gbfem_handle h, const double* b, double* x, int maxIter, cudaEvent_t ev0, cudaEvent_t ev1,
						   bool capturing = false)
{
	const int nseg = (int)h->segNode.size() - 1;
	cudaStream_t st = h->stream;
	GB_CUDA(h, cudaMemsetAsync(h->d_seg.p, 0, sizeof(SegCtl) * nseg, st));
	GB_CUDA(h, cudaMemsetAsync(h->d_pcgGlobal.p, 0, sizeof(PcgGlobal), st));
	PcgArgs a;
	a.nchunks = h->nchunks;
	a.nsegs = nseg;
	// Without an explicit cg_max_iterations every segment stops at its own default cap.
	const bool segCaps = h->prm.cg_max_iterations <= 0;
	a.maxIter = segCaps ? h->segMaxIterMax : maxIter;
	a.segMaxIter = segCaps ? h->d_segMaxIter.p : nullptr;
	a.tol = h->prm.cg_tolerance;
	// Refresh when |r|^2 has dropped 1e5x (the residual norm ~300x) since the last refresh: FP32 CG keeps
	// several digits of headroom below that, and each refresh is an FP64 pass (9 FP64 FMAs a block).
	// Measured on the 256-mesh batch: 1e-3 -> 1e-5 kept the CG iterations (226.7 / 227.1 per step)
	// and the error against the FP64 path, and cut the step by 7%.
	a.drop = 1e-5;
	a.off = h->d_off.p;
	a.col = h->d_rcol.p;
	a.val = h->d_A32.p;
	a.perm = h->d_perm.p;
	a.segChunk = h->d_segChunk.p;
	a.b = b;
	a.invdiag = h->d_invdiag32.p;
	a.x = x;
	a.brs = h->d_brs.p;
	a.r64 = h->d_r64.p;
	a.xhl = reinterpret_cast<float2*>(h->d_x64.p);  // 8 bytes per dof: one float pair
	a.xd = h->d_xd.p;
	a.invd = h->d_invd.p;
	a.r = h->d_r32.p;
	a.pA = h->d_pA.p;
	a.pB = h->d_pB.p;
	a.q = h->d_q32.p;
	a.pdir = h->d_q32.p;  // the one-phase schedule keeps p where the two-phase one keeps q
	a.cumW = h->d_cumW.p;
	a.slots = h->d_slots.p;
	a.maxChunksPerCta = h->maxChunksPerCta;
	a.refreshWeight = h->refreshWeight;
	a.pad = 0;
	a.barrierTimeoutNs = kBarrierTimeoutNs;
	a.seg = h->d_seg.p;
	a.g = h->d_pcgGlobal.p;
	a.val64 = h->d_A.p;  // FP64 batches (k_pcg_persistent<true>)
	a.invdiag64 = h->d_invdiag.p;
	a.invd64 = h->d_invd64.p;
	a.x64 = h->d_x64.p;
	a.q64 = h->d_q64.p;
	a.zA64 = h->d_zA64.p;
	a.zB64 = h->d_zB64.p;
	const unsigned evFlags = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
	if (ev0) GB_CUDA(h, cudaEventRecordWithFlags(ev0, st, evFlags));
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = dim3(h->pcgGrid);
	cfg.blockDim = dim3(kPcgThreads);
	cfg.dynamicSmemBytes = h->pcgSmem;
	cfg.stream = st;
	cudaLaunchAttribute attr[1];
	attr[0].id = cudaLaunchAttributeCooperative;  // all blocks co-resident (the grid barrier needs it)
	attr[0].val.cooperative = 1;
	cfg.attrs = attr;
	cfg.numAttrs = 1;
	GB_CUDA(h, pcg_launch(h->mixed() ? h->cgSchedule : kPcgF64, cfg, a));
	if (ev1) GB_CUDA(h, cudaEventRecordWithFlags(ev1, st, evFlags));
	h->launches += 1;
	return GBFEM_OK;
}

// Mixed-precision solve: one persistent launch, then its per-segment results are read back.
gbfem_status run_mixed(gbfem_handle h, const double* b, double* x, int maxIter, bool timeSolve)
{
	const int nseg = (int)h->segNode.size() - 1;
	cudaStream_t st = h->stream;
	static thread_local KernelTimer kt;
	if (timeSolve && !kt.init()) return fail(h, GBFEM_CUDA_ERROR, "cudaEventCreate failed");
	gbfem_status es = enqueue_mixed(h, b, x, maxIter, timeSolve ? kt.a[0] : nullptr, timeSolve ? kt.b[0] : nullptr);
	if (es != GBFEM_OK) return es;
	PcgGlobal g;
	GB_CUDA(h, cudaMemcpyAsync(h->h_seg, h->d_seg.p, sizeof(SegCtl) * nseg, cudaMemcpyDeviceToHost, st));
	GB_CUDA(h, cudaMemcpyAsync(&g, h->d_pcgGlobal.p, sizeof(PcgGlobal), cudaMemcpyDeviceToHost, st));
	GB_CUDA(h, cudaStreamSynchronize(st));
	if (g.err)
		return fail(h, GBFEM_CUDA_ERROR, g.err == 1 ? "persistent CG: grid barrier timed out"
												  : "persistent CG: work share exceeded its shared-memory bound");
	if (timeSolve)
	{
		float ms = 0;
		cudaEventElapsedTime(&ms, kt.a[0], kt.b[0]);
		h->stats.ms_spmv += ms;  // the whole persistent solve: one launch
		h->stats.spmv_timed += 1;
	}
	return GBFEM_OK;
}

// Reads the persistent solve's error flag after a synchronising point.
gbfem_status check_pcg_error(gbfem_handle h)
{
	PcgGlobal g;
	GB_CUDA(h, cudaMemcpy(&g, h->d_pcgGlobal.p, sizeof(PcgGlobal), cudaMemcpyDeviceToHost));
	if (g.err)
		return fail(h, GBFEM_CUDA_ERROR, g.err == 1 ? "persistent CG: grid barrier timed out"
												  : "persistent CG: work share exceeded its shared-memory bound");
	return GBFEM_OK;
}

// Hexahedra: the step's right-hand side from the stored K and block masses (x_t, v_t: the state the
// step started from; the current iterate is the handle's v).
void enqueue_hex_rhs(gbfem_handle h, double dt, const double* xt, const double* vt, cudaStream_t s)
{
	const MatSell3 K{h->nrows, h->d_perm.p, h->d_off.p, h->d_sellcol.p, h->d_K.p};
	if (h->mixed())
		launch_hex_rhs_df(K, h->d_Kp.p, h->d_Msp.p, h->body(), xt, h->d_v.p, vt, dt, h->prm.rayleigh_mass,
						  h->prm.rayleigh_stiffness, h->prm.gravity, h->prm.gravity_enabled, h->d_uw.p, h->d_rhs.p, s);
	else
		launch_hex_rhs(K, h->d_Ms.p, h->body(), xt, h->d_v.p, vt, dt, h->prm.rayleigh_mass, h->prm.rayleigh_stiffness,
					   h->prm.gravity, h->prm.gravity_enabled, h->d_uw.p, h->d_rhs.p, s);
}

// Autotuner of the mixed form, run on the first step's own system: times the element kernel at 32
// and 64 elements per block, then the persistent solve for 2, 3 and 4 CTAs per SM and refresh
// weights 1 to 4, and keeps the fastest of each. The element kernel's results do not depend on
// its block size; the solve's partition does change its rounding (not its convergence test), so a
// run that must reproduce another bit for bit pins the choice with gbfem_set_tuning.
gbfem_status tune_mixed(gbfem_handle h, const double* xt, const double* vt, double dt, double c1, double c2,
						int maxIter)
{
	const DevBody body = h->body();
	cudaStream_t s = h->stream;
	const double alpha = h->prm.rayleigh_mass, beta = h->prm.rayleigh_stiffness;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	GB_CUDA(h, cudaEventCreate(&e0));
	GB_CUDA(h, cudaEventCreate(&e1));
	float t = 0.f;
	auto elapsed = [&]() -> cudaError_t {
		cudaError_t e = cudaEventSynchronize(e1);
		if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
		return e;
	};
	// Element kernel: the candidates alternate; the first round warms up, the best of the next three
	// counts for each.
	float bestE32 = 1e30f, bestE64 = 1e30f;
	// FP64 batches are tuned after their step's FP64 assembly (the system is in place): only the
	// solve's CTAs per SM.
	const bool f64 = !h->mixed();
	for (int rep = 0; rep < 4 && !h->hex() && !f64; ++rep)
		for (int ept : {32, 64})
		{
			GB_CUDA(h, cudaEventRecord(e0, s));
			launch_element_f32(body, h->d_x.p, h->d_v.p, xt, vt, dt, alpha, beta, h->d_kslots32.p, h->d_rhsE32.p,
							   h->d_counters.p, s, ept, h->linear());
			GB_CUDA(h, cudaGetLastError());
			GB_CUDA(h, cudaEventRecord(e1, s));
			GB_CUDA(h, elapsed());
			float& best = (ept == 32) ? bestE32 : bestE64;
			if (rep > 0) best = std::min(best, t);
			if (rep > 0 && getenv("GBFEM_TUNE_LOG"))
				fprintf(stderr, "[gbfem tune] element kernel %d elements per block: %.3f ms\n", ept, t);
		}
	if (!h->hex() && !f64) h->elemsPerBlock = (bestE32 < bestE64) ? 32 : 64;
	if (f64)
		;  // the step's FP64 system and right-hand side are already assembled
	else if (h->hex())
	{
		launch_system_from_k(body, h->d_K.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
		enqueue_hex_rhs(h, dt, xt, vt, s);
	}
	else
	{
		launch_element_f32(body, h->d_x.p, h->d_v.p, xt, vt, dt, alpha, beta, h->d_kslots32.p, h->d_rhsE32.p,
						   h->d_counters.p, s, h->elemsPerBlock, h->linear());
		launch_assemble(body, h->d_kslots32.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
		launch_rhs_gather(body, h->d_rhsE32.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
	}
	GB_CUDA(h, cudaGetLastError());
	float bestS = 1e30f;
	int cBest = h->ctasPerSM, rBest = h->refreshWeight, fBest = h->cgSchedule;
	for (int form : {kPcgMixed2, kPcgMixed1})
	{
		if (f64 && form != kPcgMixed1) continue;  // FP64 batches have one schedule
		if (!f64) h->cgSchedule = form;
		for (int cps : {2, 3, 4})
		{
			for (int rw : {1, 2, 3, 4})
			{
				if (f64 && rw != kRefreshWeightDefault) continue;  // the FP64 solve has no refreshes
				h->refreshWeight = rw;
				if (configure_pcg(h, cps) != GBFEM_OK)
				{
					(void)cudaGetLastError();  // an infeasible candidate is skipped; clear any error it left
					continue;
				}
				gbfem_status st = enqueue_mixed(h, h->d_rhs.p, h->d_dv.p, maxIter, e0, e1);
				if (st != GBFEM_OK) return st;
				GB_CUDA(h, elapsed());
				st = check_pcg_error(h);
				if (st != GBFEM_OK) return st;
				if (getenv("GBFEM_TUNE_LOG"))
					fprintf(stderr, "[gbfem tune] schedule %d ctas/SM %d refresh weight %d: %.3f ms\n", form, cps, rw, t);
				if (t < bestS)
				{
					bestS = t;
					cBest = cps;
					rBest = rw;
					fBest = form;
				}
			}
		}
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (!f64) h->cgSchedule = fBest;
	h->refreshWeight = rBest;
	gbfem_status st = configure_pcg(h, cBest);
	if (st != GBFEM_OK) return st;
	h->tuned = true;
	h->tuneVersion++;
	h->err.clear();
	if (!f64) GB_CUDA(h, cudaMemsetAsync(h->d_counters.p, 0, 4 * sizeof(int), s));  // count the real step only
	return GBFEM_OK;
}

// One mixed-form step (first Newton iteration) enqueued without host synchronisation, then the
// per-segment statistics accumulated on the device: the body of the captured step graph.
gbfem_status enqueue_step_mixed(gbfem_handle h, double dt, bool timed)
{
	const DevBody body = h->body();
	cudaStream_t s = h->stream;
	const Launch L = h->launch();
	const int nseg = (int)h->segNode.size() - 1;
	const int maxIter = h->stepMaxIter();
	const double c1 = 1.0 / dt + h->prm.rayleigh_mass, c2 = dt + h->prm.rayleigh_stiffness;
	const bool reuse = h->systemCurrent(dt);
	int kernels = 0;
	if (!h->mixed())
	{
		// FP64 batch: the FP64 element update and assembly, then the persistent FP64 solve.
		if (h->hex())
		{
			if (!reuse) launch_system_from_k(body, h->d_K.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
			enqueue_hex_rhs(h, dt, h->d_x.p, h->d_v.p, s);
			kernels = reuse ? 2 : 3;
		}
		else
		{
			launch_element_fp64(body, h->d_x.p, h->d_v.p, h->d_x.p, h->d_v.p, dt, h->prm.rayleigh_mass,
								h->prm.rayleigh_stiffness, reuse ? nullptr : h->d_kslots.p, h->d_rhsE.p, nullptr, nullptr,
								h->d_counters.p, s, h->linear());
			if (!reuse) launch_assemble(body, h->d_kslots.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
			launch_rhs_gather(body, h->d_rhsE.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
			kernels = 1 + (reuse ? 1 : 2);
		}
	}
	else if (h->hex())
	{
		if (!reuse) launch_system_from_k(body, h->d_K.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
		enqueue_hex_rhs(h, dt, h->d_x.p, h->d_v.p, s);
		kernels = reuse ? 2 : 3;
	}
	else
	{
		const int ek = launch_element_f32(body, h->d_x.p, h->d_v.p, h->d_x.p, h->d_v.p, dt, h->prm.rayleigh_mass,
										  h->prm.rayleigh_stiffness, reuse ? nullptr : h->d_kslots32.p,
										  h->d_rhsE32.p, h->d_counters.p, s, h->elemsPerBlock, h->linear());
		if (!reuse) launch_assemble(body, h->d_kslots32.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
		launch_rhs_gather(body, h->d_rhsE32.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
		kernels = ek + (reuse ? 1 : 2);
	}
	gbfem_status st = enqueue_mixed(h, h->d_rhs.p, h->d_dv.p, maxIter, timed ? h->graphEv[0] : nullptr,
									timed ? h->graphEv[1] : nullptr, /*capturing=*/true);
	if (st != GBFEM_OK) return st;
	launch_state_update(h->n, h->d_dv.p, h->d_dvPrev.p, h->d_x.p, h->d_x.p, h->d_v.p, dt, 0, h->d_ctl.p, h->d_part.p, L);
	launch_validity(h->n, h->d_x.p, h->d_v.p, h->d_ctl.p, h->d_part.p, L);
	launch_step_accumulate(h->d_seg.p, nseg, &h->d_ctl.p->nonfinite, &h->d_pcgGlobal.p->err, h->d_acc.p, s);
	GB_CUDA(h, cudaGetLastError());
	h->graphKernels = kernels + 4;  // + solve, state update, validity, accumulate
	return GBFEM_OK;
}

// GBFEM_STEP_GRAPH: the step is captured once into a CUDA graph (per dt, timing flag and tuning)
// and the graph is launched nsteps times with no host round trip between steps; statistics and the
// finiteness check are accumulated on the device and read once at the end.
gbfem_status step_graph(gbfem_handle h, double dt, int nsteps, uint32_t flags)
{
	if (!h->persistent() || h->prm.newton_max_iterations > 1 || (flags & GBFEM_STEP_KEEP_SYSTEM))
		return fail(h, GBFEM_INVALID_ARG,
					"GBFEM_STEP_GRAPH needs the mixed form or a batch, one Newton iteration and no GBFEM_STEP_KEEP_SYSTEM");
	cudaStream_t s = h->stream;
	const int nseg = (int)h->segNode.size() - 1;
	const bool timed = (flags & GBFEM_STEP_TIME_KERNELS) != 0;
	if (!h->graphExec || h->graphDt != dt || h->graphTimed != timed || h->graphVersion != h->tuneVersion)
	{
		if (h->graphExec) cudaGraphExecDestroy(h->graphExec);
		h->graphExec = nullptr;
		if (timed && !h->graphEv[0])
		{
			GB_CUDA(h, cudaEventCreate(&h->graphEv[0]));
			GB_CUDA(h, cudaEventCreate(&h->graphEv[1]));
		}
		GB_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		const int launchesBefore = h->launches;
		gbfem_status st = enqueue_step_mixed(h, dt, timed);
		h->launches = launchesBefore;
		cudaGraph_t graph = nullptr;
		const cudaError_t ce = cudaStreamEndCapture(s, &graph);
		if (st != GBFEM_OK)
		{
			if (graph) cudaGraphDestroy(graph);
			return st;
		}
		GB_CUDA(h, ce);
		const cudaError_t ie = cudaGraphInstantiate(&h->graphExec, graph, 0);
		cudaGraphDestroy(graph);
		GB_CUDA(h, ie);
		h->graphDt = dt;
		h->graphTimed = timed;
		h->graphVersion = h->tuneVersion;
	}
	std::vector<double> acc(4 * (size_t)nseg + 2, 0.0);
	for (int k = 0; k < nseg; ++k) acc[4 * (size_t)k + 2] = 1.0;
	GB_CUDA(h, cudaMemcpyAsync(h->d_acc.p, acc.data(), sizeof(double) * acc.size(), cudaMemcpyHostToDevice, s));
	GB_CUDA(h, cudaMemsetAsync(h->d_pcgGlobal.p, 0, sizeof(PcgGlobal), s));
	for (int i = 0; i < nsteps; ++i)
	{
		GB_CUDA(h, cudaGraphLaunch(h->graphExec, s));
		h->launches += h->graphKernels;
		if (timed)
		{
			GB_CUDA(h, cudaStreamSynchronize(s));
			float ms = 0.f;
			GB_CUDA(h, cudaEventElapsedTime(&ms, h->graphEv[0], h->graphEv[1]));
			h->stats.ms_spmv += ms;
			h->stats.spmv_timed += 1;
		}
	}
	GB_CUDA(h, cudaMemcpyAsync(acc.data(), h->d_acc.p, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, s));
	GB_CUDA(h, cudaStreamSynchronize(s));
	GB_CUDA(h, cudaGetLastError());
	double worst = 0.0;
	for (int k = 0; k < nseg; ++k)
	{
		const double* a = &acc[4 * (size_t)k];
		h->stats.cg_iterations += (int)a[0];
		h->stats.refinement_sweeps += (int)a[1];
		if (a[2] < 1.0) h->stats.cg_max_iterations_hit++;
		worst = std::max(worst, a[3]);
		double* ss = &h->segStats[4 * (size_t)k];
		ss[0] += a[0];
		ss[1] += a[1];
		ss[2] = std::min(ss[2], a[2]);
		ss[3] = std::max(ss[3], a[3]);
	}
	h->stats.cg_relative_residual = worst;
	h->stats.steps += nsteps;
	h->systemReady = true;
	h->lastDt = dt;
	if (acc[4 * (size_t)nseg + 1] != 0.0) return fail(h, GBFEM_CUDA_ERROR, "persistent CG: grid barrier timed out");
	if (acc[4 * (size_t)nseg] != 0.0)
	{
		h->active = false;  // FemRepresentation.cpp:285-293
		return fail(h, GBFEM_NONFINITE, "state is not finite after a graph-launched step; representation deactivated");
	}
	return GBFEM_OK;
}

// Applies the pending external generalized forces after the step's assembly (FemRepresentation::
// computeFMDK, FemRepresentation.cpp:527-544: f += F_ext, K += K_ext, D += D_ext): S gains D + dt K on
// the lower blocks the CG reads, the right-hand side F + K (x_n - x_t - dt v_n), both skipping
// boundary-condition rows and columns. Two launches.
gbfem_status apply_external(gbfem_handle h, double dt, const double* xt, cudaStream_t s)
{
	const int N = h->N;
	std::vector<ExtBlock> blocks;
	std::vector<ExtRow> rows;
	std::vector<ExtCol> cols;
	std::vector<char> rowSeen(N, 0);
	auto row_of = [&](int I) -> ExtRow& {
		if (rows.empty() || rows.back().I != I)
		{
			ExtRow r{};
			r.I = I;
			r.k0 = r.k1 = (int)cols.size();
			for (int i = 0; i < 3; ++i) r.F[i] = h->extF[3 * (size_t)I + i];
			rows.push_back(r);
			rowSeen[I] = 1;
		}
		return rows.back();
	};
	for (const auto& kv : h->extBlocks)  // keys in (I, J) order
	{
		const int I = (int)(kv.first / N), J = (int)(kv.first % N);
		const auto& v = kv.second;
		ExtRow& r = row_of(I);
		ExtCol c{};
		c.J = J;
		for (int k = 0; k < 9; ++k) c.K[k] = v[k];
		cols.push_back(c);
		r.k1 = (int)cols.size();
		if (I >= J)
		{
			const int pos = h->blockPos(I, J);
			const int L = pos >= 0 ? h->lowerOfPosHost[pos] : -1;
			if (L < 0) return fail(h, GBFEM_CUDA_ERROR, "internal error: external block outside the pattern");
			ExtBlock b{};
			b.z = h->lblkHost[L].z;
			b.w = h->lblkHost[L].w;
			b.I = I;
			b.J = J;
			for (int k = 0; k < 9; ++k) b.v[k] = v[9 + k] + dt * v[k];
			blocks.push_back(b);
		}
	}
	for (int I = 0; I < N; ++I)  // nodes with a force and no external block
		if (!rowSeen[I] && (h->extF[3 * (size_t)I] != 0.0 || h->extF[3 * (size_t)I + 1] != 0.0 ||
							h->extF[3 * (size_t)I + 2] != 0.0))
		{
			ExtRow r{};
			r.I = I;
			r.k0 = r.k1 = 0;
			for (int i = 0; i < 3; ++i) r.F[i] = h->extF[3 * (size_t)I + i];
			rows.push_back(r);
		}
	const size_t bB = sizeof(ExtBlock) * blocks.size(), bR = sizeof(ExtRow) * rows.size(), bC = sizeof(ExtCol) * cols.size();
	const size_t total = bB + bR + bC;
	if (total == 0) return GBFEM_OK;
	if (h->d_ext.n < total) GB_CUDA(h, h->d_ext.alloc(total));
	std::vector<unsigned char> pack(total);
	std::memcpy(pack.data(), blocks.data(), bB);
	std::memcpy(pack.data() + bB, rows.data(), bR);
	std::memcpy(pack.data() + bB + bR, cols.data(), bC);
	GB_CUDA(h, cudaMemcpyAsync(h->d_ext.p, pack.data(), total, cudaMemcpyHostToDevice, s));
	const ExtBlock* dB = reinterpret_cast<const ExtBlock*>(h->d_ext.p);
	const ExtRow* dR = reinterpret_cast<const ExtRow*>(h->d_ext.p + bB);
	const ExtCol* dC = reinterpret_cast<const ExtCol*>(h->d_ext.p + bB + bR);
	if (h->mixed())
		launch_ext_system((int)blocks.size(), dB, h->d_bc.p, h->d_A32.p, h->d_invdiag32.p, s);
	else
		launch_ext_system((int)blocks.size(), dB, h->d_bc.p, h->d_A.p, h->d_invdiag.p, s);
	launch_ext_rhs((int)rows.size(), dR, dC, h->d_bc.p, h->d_x.p, xt, h->d_v.p, dt, h->d_rhs.p, s);
	GB_CUDA(h, cudaGetLastError());
	GB_CUDA(h, cudaStreamSynchronize(s));  // the host pack is released on return
	h->launches += 2;
	return GBFEM_OK;
}

// Per-segment results of the last persistent solve (read back by run_mixed) into the statistics.
void collect_segment_stats(gbfem_handle h)
{
	double worst = 0.0;
	for (int sg = 0; sg + 1 < (int)h->segNode.size(); ++sg)
	{
		const SegCtl& c = h->h_seg[sg];
		const double res = c.bb > 0 ? std::sqrt(c.rrTrue / c.bb) : 0.0;
		h->stats.cg_iterations += c.iter;
		h->stats.refinement_sweeps += c.updates;
		worst = std::max(worst, res);
		if (!c.converged) h->stats.cg_max_iterations_hit++;
		double* ss = &h->segStats[4 * (size_t)sg];
		ss[0] += c.iter;
		ss[1] += c.updates;
		ss[2] = std::min(ss[2], (double)c.converged);
		ss[3] = std::max(ss[3], res);
	}
	h->stats.cg_relative_residual = worst;
}

gbfem_status step_once(gbfem_handle h, double dt, uint32_t flags)
{
	const bool keep = (flags & GBFEM_STEP_KEEP_SYSTEM) != 0;
	if (keep && h->mixed())
		return fail(h, GBFEM_INVALID_ARG, "GBFEM_STEP_KEEP_SYSTEM is available in the FP64 form only");
	if (keep && h->hex()) return fail(h, GBFEM_INVALID_ARG, "GBFEM_STEP_KEEP_SYSTEM is available for tetrahedra only");
	if (keep && h->extActive)
		return fail(h, GBFEM_INVALID_ARG, "GBFEM_STEP_KEEP_SYSTEM does not export external forces");
	if (keep)
	{
		gbfem_status st = ensure_system_maps(h);
		if (st != GBFEM_OK) return st;
	}
	const Launch L = h->launch();
	cudaStream_t s = h->stream;
	const DevBody body = h->body();
	const int newtonMax = std::max(1, (int)h->prm.newton_max_iterations);
	const int maxIter = h->stepMaxIter();
	const double c1 = 1.0 / dt + h->prm.rayleigh_mass;
	const double c2 = dt + h->prm.rayleigh_stiffness;
	double* xt = h->d_x.p;
	double* vt = h->d_v.p;
	if (newtonMax > 1)
	{
		if (!h->d_xt.p)
		{
			GB_CUDA(h, h->d_xt.alloc(h->n));
			GB_CUDA(h, h->d_vt.alloc(h->n));
			GB_CUDA(h, h->d_dvPrev.alloc(h->n));
		}
		GB_CUDA(h, cudaMemcpyAsync(h->d_xt.p, h->d_x.p, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, s));
		GB_CUDA(h, cudaMemcpyAsync(h->d_vt.p, h->d_v.p, sizeof(double) * h->n, cudaMemcpyDeviceToDevice, s));
		GB_CUDA(h, cudaMemsetAsync(h->d_dvPrev.p, 0, sizeof(double) * h->n, s));
		xt = h->d_xt.p;
		vt = h->d_vt.p;
	}
	PhaseTimer tm;
	tm.init((flags & GBFEM_STEP_TIME_PHASES) != 0, s);
	for (int it = 0; it < newtonMax; ++it)
	{
		tm.mark(0);
		const bool timeK = (flags & GBFEM_STEP_TIME_KERNELS) != 0;
		if (h->mixed())
		{
			if (h->prm.autotune && !h->tuned)
			{
				gbfem_status tst = tune_mixed(h, xt, vt, dt, c1, c2, maxIter);
				if (tst != GBFEM_OK) return tst;
			}
			const bool reuse = h->systemCurrent(dt);
			int ek = 1;  // kernels of the element update (hexahedra: the right-hand-side pair counts as one)
			if (h->hex())
			{
				enqueue_hex_rhs(h, dt, xt, vt, s);
				tm.mark(1);
				if (!reuse) launch_system_from_k(body, h->d_K.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
			}
			else
			{
				ek = launch_element_f32(body, h->d_x.p, h->d_v.p, xt, vt, dt, h->prm.rayleigh_mass,
								   h->prm.rayleigh_stiffness, reuse ? nullptr : h->d_kslots32.p, h->d_rhsE32.p,
								   h->d_counters.p, s, h->elemsPerBlock, h->linear());
				tm.mark(1);
				if (!reuse) launch_assemble(body, h->d_kslots32.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
				launch_rhs_gather(body, h->d_rhsE32.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
			}
			if (h->constantSystem() && !reuse)
			{
				h->linearReady = true;
				h->linearDt = dt;
				h->tuneVersion++;  // a captured step graph must be rebuilt (right-hand side only from now on)
			}
			GB_CUDA(h, cudaGetLastError());
			h->launches += ek + 1 + (reuse ? 0 : 1);
			if (h->extActive)
			{
				gbfem_status est = apply_external(h, dt, xt, s);
				if (est != GBFEM_OK) return est;
			}
			tm.mark(2);
			gbfem_status st = run_mixed(h, h->d_rhs.p, h->d_dv.p, maxIter, timeK);
			if (st != GBFEM_OK) return st;
			tm.mark(3);
			collect_segment_stats(h);
		}
		else
		{
			const bool reuse = h->systemCurrent(dt) && !keep;
			if (h->hex())
			{
				enqueue_hex_rhs(h, dt, xt, vt, s);
				tm.mark(1);
				if (!reuse) launch_system_from_k(body, h->d_K.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
			}
			else
			{
				launch_element_fp64(body, h->d_x.p, h->d_v.p, xt, vt, dt, h->prm.rayleigh_mass,
									h->prm.rayleigh_stiffness, reuse ? nullptr : h->d_kslots.p, h->d_rhsE.p,
									keep ? h->d_kfull.p : nullptr, keep ? h->d_fE.p : nullptr, h->d_counters.p, s,
									h->linear());
				tm.mark(1);
				if (!reuse) launch_assemble(body, h->d_kslots.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
				launch_rhs_gather(body, h->d_rhsE.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
			}
			if (h->constantSystem() && !reuse)
			{
				h->linearReady = true;
				h->linearDt = dt;
			}
			if (keep)
			{
				launch_assemble_full_csc((int)h->nnz, h->d_sptr.p, h->d_sidx.p, h->d_srow.p, h->d_scol.p,
										 h->d_kfull.p, h->d_smass.p, h->d_bc.p, c1, c2, h->d_S.p, s);
				launch_rhs_gather(body, h->d_fE.p, h->prm.gravity, h->prm.gravity_enabled, h->d_f.p, 0, s);
			}
			GB_CUDA(h, cudaGetLastError());
			h->launches += keep ? 5 : 2 + (reuse ? 0 : 1);
			if (h->extActive)
			{
				gbfem_status est = apply_external(h, dt, xt, s);
				if (est != GBFEM_OK) return est;
			}
			tm.mark(2);
			if (h->batched())
			{
				// FP64 batch: every mesh's Eigen CG in one persistent FP64 launch.
				if (h->prm.autotune && !h->tuned)
				{
					gbfem_status tst = tune_mixed(h, xt, vt, dt, c1, c2, maxIter);
					if (tst != GBFEM_OK) return tst;
				}
				gbfem_status st = run_mixed(h, h->d_rhs.p, h->d_dv.p, maxIter, timeK);
				if (st != GBFEM_OK) return st;
				tm.mark(3);
				collect_segment_stats(h);
			}
			else
			{
				gbfem_status st = run_cg(h, h->d_rhs.p, h->d_dv.p, maxIter, timeK);
				if (st != GBFEM_OK) return st;
				tm.mark(3);
				h->stats.cg_iterations += h->h_ctl->iter;
				h->stats.cg_relative_residual = h->h_ctl->bb > 0 ? std::sqrt(h->h_ctl->rr / h->h_ctl->bb) : 0.0;
				if (!h->h_ctl->converged) h->stats.cg_max_iterations_hit++;
				h->segStats[0] += h->h_ctl->iter;
				h->segStats[2] = std::min(h->segStats[2], (double)h->h_ctl->converged);
				h->segStats[3] = std::max(h->segStats[3], h->stats.cg_relative_residual);
			}
		}
		launch_state_update(h->n, h->d_dv.p, h->d_dvPrev.p, xt, h->d_x.p, h->d_v.p, dt, newtonMax > 1, h->d_ctl.p,
							h->d_part.p, L);
		h->launches++;
		tm.mark(4);
		if (tm.on)
		{
			GB_CUDA(h, cudaStreamSynchronize(s));
			h->stats.ms_element += tm.ms(0, 1);
			h->stats.ms_assemble += tm.ms(1, 2);
			h->stats.ms_solve += tm.ms(2, 3);
			h->stats.ms_update += tm.ms(3, 4);
		}
		if (newtonMax > 1)
		{
			GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl.p, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
			GB_CUDA(h, cudaStreamSynchronize(s));
			if (h->h_ctl->newtonVar < h->prm.newton_epsilon) break;  // OdeSolverEulerImplicit.cpp:101-112
		}
	}
	h->haveSystem = keep;
	launch_validity(h->n, h->d_x.p, h->d_v.p, h->d_ctl.p, h->d_part.p, L);
	h->launches++;
	GB_CUDA(h, cudaMemcpyAsync(h->h_ctl, h->d_ctl.p, sizeof(CgCtl), cudaMemcpyDeviceToHost, s));
	GB_CUDA(h, cudaStreamSynchronize(s));
	GB_CUDA(h, cudaGetLastError());
	h->stats.steps++;
	h->systemReady = true;
	h->lastDt = dt;
	if (h->h_ctl->nonfinite)
	{
		h->active = false;  // FemRepresentation.cpp:285-293
		return fail(h, GBFEM_NONFINITE, "state is not finite; representation deactivated");
	}
	return GBFEM_OK;
}

}  // namespace

extern "C" {

gbfem_status gbfem_params_default(gbfem_params* out)
{
	if (!out) return GBFEM_INVALID_ARG;
	std::memset(out, 0, sizeof(*out));
	out->rayleigh_mass = 0.0;
	out->rayleigh_stiffness = 0.0;
	out->gravity[0] = 0.0;
	out->gravity[1] = -9.81;
	out->gravity[2] = 0.0;
	out->gravity_enabled = 1;
	out->newton_max_iterations = 1;
	out->newton_epsilon = 1e-5;
	out->cg_tolerance = DBL_EPSILON;
	out->cg_max_iterations = 0;
	out->precision = GBFEM_PRECISION_FP64;
	out->device = 0;
	return GBFEM_OK;
}

}  // extern "C"

namespace {

// Checks one mesh description (Fem3DRepresentation / FemElement / OdeState input checks).
gbfem_status validate_mesh(const gbfem_mesh_desc* m, int index, int elementType)
{
	const std::string where = index >= 0 ? "mesh " + std::to_string(index) + ": " : std::string();
	if (!m) return fail(nullptr, GBFEM_INVALID_ARG, where + "mesh is NULL");
	if (m->num_nodes <= 0 || m->num_tets <= 0 || !m->rest_positions || !m->tets || !m->young_modulus ||
		!m->poisson_ratio || !m->mass_density || (m->num_bc_dofs > 0 && !m->bc_dofs) || m->num_bc_dofs < 0)
		return fail(nullptr, GBFEM_INVALID_ARG, where + "empty mesh or missing arrays");
	if (m->num_nodes > INT32_MAX / 3) return fail(nullptr, GBFEM_INVALID_ARG, where + "too many nodes");
	const int npe = elementType == GBFEM_ELEMENT_HEXAHEDRON ? 8 : 4;
	for (int64_t i = 0; i < (int64_t)npe * m->num_tets; ++i)
		if (m->tets[i] < 0 || m->tets[i] >= m->num_nodes)
			return fail(nullptr, GBFEM_INVALID_ARG, where + "Invalid nodeId " + std::to_string(m->tets[i]));
	if (elementType == GBFEM_ELEMENT_HEXAHEDRON)
		for (int32_t e = 0; e < m->num_tets; ++e)
		{
			const int32_t* nd = m->tets + 8 * (size_t)e;
			for (int a = 0; a < 8; ++a)
				for (int b = a + 1; b < 8; ++b)
					if (nd[a] == nd[b])
						return fail(nullptr, GBFEM_INVALID_ARG, where + "hexahedron " + std::to_string(e) + " repeats a node");
			double vol = 0.0;
			const int chk = hex_rest_check(m->rest_positions, nd, &vol);
			if (chk == 1)
				return fail(nullptr, GBFEM_DEGENERATE_ELEMENT,
							where + "hexahedron " + std::to_string(e) + ": non invertible Jacobian at a Gauss point");
			if (chk == 2)
				return fail(nullptr, GBFEM_DEGENERATE_ELEMENT,
							where + "hexahedron " + std::to_string(e) + " ill-defined, its volume is " + std::to_string(vol));
		}
	for (int32_t e = 0; e < m->num_tets; ++e)
	{
		// FemElement::initialize material checks (FemElement.cpp:33-43).
		const double rho = m->mass_density[e], nu = m->poisson_ratio[e], Ey = m->young_modulus[e];
		if (!(rho > 0.0) || !(nu > 0.0 && nu < 0.5) || !(Ey > 0.0))
			return fail(nullptr, GBFEM_INVALID_ARG, where + "invalid material on element " + std::to_string(e));
	}
	for (int32_t i = 0; i < m->num_bc_dofs; ++i)
		if (m->bc_dofs[i] < 0 || m->bc_dofs[i] >= 3 * m->num_nodes)
			return fail(nullptr, GBFEM_INVALID_ARG,
						where + "Invalid boundary condition dof " + std::to_string(m->bc_dofs[i]));
	return GBFEM_OK;
}

gbfem_status create_impl(const gbfem_mesh_desc* meshes, int32_t count, const gbfem_params* prm, gbfem_handle* out)
{
	if (!out) return fail(nullptr, GBFEM_INVALID_ARG, "out is NULL");
	*out = nullptr;
	if (!meshes || !prm || count <= 0) return fail(nullptr, GBFEM_INVALID_ARG, "mesh or params is NULL");
	if (!(prm->newton_max_iterations >= 1) || !(prm->newton_epsilon >= 0.0) || !(prm->cg_tolerance >= 0.0) ||
		prm->precision < 0 || prm->precision > 1 || prm->element_type < 0 || prm->element_type > 2 ||
		prm->mass_lumping < 0 || prm->mass_lumping > 1)
		return fail(nullptr, GBFEM_INVALID_ARG, "invalid solver parameters");
	for (int32_t k = 0; k < count; ++k)
	{
		gbfem_status st = validate_mesh(&meshes[k], count > 1 ? k : -1, prm->element_type);
		if (st != GBFEM_OK) return st;
	}
	const int npe = prm->element_type == GBFEM_ELEMENT_HEXAHEDRON ? 8 : 4;
	const int slotsPerElement = prm->element_type == GBFEM_ELEMENT_HEXAHEDRON ? kHexSlots : kSlots;
	// Concatenate the meshes (node ids, boundary-condition dofs shifted by the node offsets).
	int64_t N = 0, E = 0, B = 0;
	for (int32_t k = 0; k < count; ++k)
	{
		N += meshes[k].num_nodes;
		E += meshes[k].num_tets;
		B += meshes[k].num_bc_dofs;
	}
	if (N > INT32_MAX / 3 || E > INT32_MAX / slotsPerElement) return fail(nullptr, GBFEM_INVALID_ARG, "batch too large");
	std::vector<double> X, Ey, Nu, Rho;
	std::vector<int32_t> T, Bc;
	std::vector<int> segNode{0}, segTet{0};
	if (count > 1)
	{
		X.reserve(3 * N);
		T.reserve(npe * E);
		Ey.reserve(E);
		Nu.reserve(E);
		Rho.reserve(E);
		Bc.reserve(B);
	}
	for (int32_t k = 0; k < count; ++k)
	{
		const gbfem_mesh_desc& m = meshes[k];
		const int32_t n0 = segNode.back();
		if (count > 1)
		{
			X.insert(X.end(), m.rest_positions, m.rest_positions + 3 * (size_t)m.num_nodes);
			for (int64_t i = 0; i < (int64_t)npe * m.num_tets; ++i) T.push_back(m.tets[i] + n0);
			Ey.insert(Ey.end(), m.young_modulus, m.young_modulus + m.num_tets);
			Nu.insert(Nu.end(), m.poisson_ratio, m.poisson_ratio + m.num_tets);
			Rho.insert(Rho.end(), m.mass_density, m.mass_density + m.num_tets);
			for (int32_t i = 0; i < m.num_bc_dofs; ++i) Bc.push_back(m.bc_dofs[i] + 3 * n0);
		}
		segNode.push_back(n0 + m.num_nodes);
		segTet.push_back(segTet.back() + m.num_tets);
	}
	gbfem_mesh_desc merged = meshes[0];
	if (count > 1)
		merged = gbfem_mesh_desc{(int32_t)N, X.data(), (int32_t)E, T.data(), Ey.data(), Nu.data(), Rho.data(),
								 (int32_t)B, Bc.data()};
	auto* h = new gbfem_handle_s();
	h->prm = *prm;
	h->device = prm->device;
	h->segNode = segNode;
	h->segTet = segTet;
	cudaError_t ce = cudaSetDevice(h->device);
	if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
	if (ce != cudaSuccess)
	{
		std::string msg = std::string("CUDA unavailable: ") + cudaGetErrorString(ce);
		delete h;
		return fail(nullptr, GBFEM_CUDA_ERROR, msg);
	}
	gbfem_status st = build_body(h, &merged);
	if (st != GBFEM_OK)
	{
		g_lastCreateError = h->err;
		h->release();
		delete h;
		return st;
	}
	h->stats.active = 1;
	h->segStats.assign(4 * (size_t)count, 0.0);
	*out = h;
	return GBFEM_OK;
}

}  // namespace

extern "C" {

gbfem_status gbfem_create(const gbfem_mesh_desc* m, const gbfem_params* prm, gbfem_handle* out)
{
	return create_impl(m, 1, prm, out);
}

gbfem_status gbfem_batch_create(int32_t count, const gbfem_mesh_desc* meshes, const gbfem_params* params,
								gbfem_handle* out)
{
	return create_impl(meshes, count, params, out);
}

gbfem_status gbfem_apply_compliance(gbfem_handle h, int32_t ncols, const double* b, double* x, uint32_t flags,
									int32_t* iterations)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (ncols < 0 || (ncols > 0 && (!b || !x))) return fail(h, GBFEM_INVALID_ARG, "gbfem_apply_compliance: bad arrays");
	if (!h->systemReady) return fail(h, GBFEM_INVALID_ARG, "gbfem_apply_compliance: no step has assembled a system yet");
	const bool warp = (flags & GBFEM_COMPLIANCE_WARPING) != 0;
	if (warp && !h->corotational())
		return fail(h, GBFEM_INVALID_ARG, "compliance warping needs the corotational element");
	GB_CUDA(h, cudaSetDevice(h->device));
	const int n = h->n, N = h->N;
	const Launch L = h->launch();
	cudaStream_t s = h->stream;
	const size_t n8 = (size_t)n * kMcgCols;
	if (!h->d_mcgVec.p)
	{
		GB_CUDA(h, h->d_mcgVec.alloc(6 * n8));
		GB_CUDA(h, h->d_mcgPart.alloc(2 * (size_t)kMcgCols * L.vecGrid));
		GB_CUDA(h, h->d_mcgCtl.alloc(1));
		GB_CUDA(h, cudaMemsetAsync(h->d_mcgCtl.p, 0, sizeof(McgCtl), s));
		GB_CUDA(h, cudaMallocHost(&h->h_mcgCtl, sizeof(McgCtl)));
	}
	const DevBody body = h->body();
	if (warp)
	{
		if (!h->d_Re.p)
		{
			GB_CUDA(h, h->d_Re.alloc(9 * (size_t)h->E));
			GB_CUDA(h, h->d_Wn.alloc(9 * (size_t)N));
			GB_CUDA(h, h->d_xprev.alloc(n));
		}
		// The rotations of the last element update: at the positions the last step started from.
		launch_prev_positions(n, h->d_x.p, h->d_v.p, h->lastDt, h->d_xprev.p, s);
		launch_element_rotation(body, h->d_xprev.p, h->d_Re.p, s);
		launch_node_rotation(body, h->d_Re.p, h->d_Wn.p, s);
	}
	double *B = h->d_mcgVec.p, *X = B + n8, *R = X + n8, *Z = R + n8, *P = Z + n8, *Q = P + n8;
	const MatSellT<double> A64{h->nrows, h->d_perm.p, h->d_off.p, h->d_sellcol.p, h->d_A.p};
	const MatSellT<float> A32{h->nrows, h->d_perm.p, h->d_off.p, h->d_sellcol.p, h->d_A32.p};
	const bool m32 = h->mixed();
	const int maxIter = h->prm.cg_max_iterations > 0 ? h->prm.cg_max_iterations : 2 * n;
	std::vector<double> hb(n8);
	int totalIt = 0;
	bool allConverged = true;
	for (int c0 = 0; c0 < ncols; c0 += kMcgCols)
	{
		const int k = std::min(kMcgCols, ncols - c0);
		std::fill(hb.begin(), hb.end(), 0.0);
		for (int c = 0; c < k; ++c)
			for (int i = 0; i < n; ++i) hb[(size_t)i * kMcgCols + c] = b[(size_t)(c0 + c) * n + i];
		GB_CUDA(h, cudaMemcpyAsync(B, hb.data(), sizeof(double) * n8, cudaMemcpyHostToDevice, s));
		if (warp) launch_apply_node_rotation(N, h->d_Wn.p, B, true, s);
		launch_mcg_init(n, k, B, h->d_bc.p, m32 ? nullptr : h->d_invdiag.p, m32 ? h->d_invdiag32.p : nullptr, X, R, Z,
						P, h->d_mcgCtl.p, h->d_mcgPart.p, h->prm.cg_tolerance, maxIter, L);
		GB_CUDA(h, cudaGetLastError());
		int chunk = 8;
		for (long long done = 0;; done += chunk)
		{
			for (int j = 0; j < chunk; ++j)
			{
				launch_mcg_spmm(m32 ? nullptr : &A64, m32 ? &A32 : nullptr, P, Q, h->d_mcgCtl.p, h->d_mcgPart.p, L);
				launch_mcg_update(n, m32 ? nullptr : h->d_invdiag.p, m32 ? h->d_invdiag32.p : nullptr, P, Q, X, R, Z,
								  h->d_mcgCtl.p, h->d_mcgPart.p, L);
				launch_mcg_pupdate(n, Z, P, h->d_mcgCtl.p, L);
			}
			GB_CUDA(h, cudaGetLastError());
			GB_CUDA(h, cudaMemcpyAsync(h->h_mcgCtl, h->d_mcgCtl.p, sizeof(McgCtl), cudaMemcpyDeviceToHost, s));
			GB_CUDA(h, cudaStreamSynchronize(s));
			if (h->h_mcgCtl->allDone) break;
			if (done > (long long)maxIter + 64) return fail(h, GBFEM_CUDA_ERROR, "compliance CG control block did not finish");
			chunk = std::min(2 * chunk, 64);
		}
		if (warp) launch_apply_node_rotation(N, h->d_Wn.p, X, false, s);
		GB_CUDA(h, cudaMemcpyAsync(hb.data(), X, sizeof(double) * n8, cudaMemcpyDeviceToHost, s));
		GB_CUDA(h, cudaStreamSynchronize(s));
		for (int c = 0; c < k; ++c)
		{
			for (int i = 0; i < n; ++i) x[(size_t)(c0 + c) * n + i] = hb[(size_t)i * kMcgCols + c];
			totalIt += h->h_mcgCtl->iter[c];
			allConverged = allConverged && h->h_mcgCtl->converged[c];
		}
	}
	if (iterations) *iterations = totalIt;
	return allConverged ? GBFEM_OK : fail(h, GBFEM_CG_MAXITER, "a compliance column did not converge");
}

gbfem_status gbfem_get_tuning(gbfem_handle h, int32_t* elems_per_block, int32_t* ctas_per_sm, int32_t* refresh_weight,
							  int32_t* cg_schedule)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (elems_per_block) *elems_per_block = h->elemsPerBlock;
	if (ctas_per_sm) *ctas_per_sm = h->ctasPerSM;
	if (refresh_weight) *refresh_weight = h->refreshWeight;
	if (cg_schedule) *cg_schedule = h->mixed() ? h->cgSchedule : kPcgF64;
	return GBFEM_OK;
}

gbfem_status gbfem_set_tuning(gbfem_handle h, int32_t elems_per_block, int32_t ctas_per_sm, int32_t refresh_weight,
							  int32_t cg_schedule)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!h->persistent()) return fail(h, GBFEM_INVALID_ARG, "tuning applies to the mixed form and to batches");
	if ((elems_per_block != 32 && elems_per_block != 64) || ctas_per_sm < 1 || ctas_per_sm > 4 || refresh_weight < 1 ||
		refresh_weight > kRefreshWeightMax)
		return fail(h, GBFEM_INVALID_ARG, "tuning: elems_per_block 32|64, ctas_per_sm 1..4, refresh_weight 1..8");
	const bool mixedSchedule = cg_schedule == GBFEM_CG_TWO_PHASE || cg_schedule == GBFEM_CG_ONE_PHASE;
	if (cg_schedule >= 0 && (h->mixed() ? !mixedSchedule : cg_schedule != GBFEM_CG_FP64))
		return fail(h, GBFEM_INVALID_ARG, "tuning: cg_schedule must be -1 (keep), GBFEM_CG_TWO_PHASE or GBFEM_CG_ONE_PHASE "
										  "(mixed form), GBFEM_CG_FP64 (FP64 batches)");
	GB_CUDA(h, cudaSetDevice(h->device));
	const int oldSchedule = h->cgSchedule, oldWeight = h->refreshWeight;
	if (h->mixed() && cg_schedule >= 0) h->cgSchedule = cg_schedule;
	h->refreshWeight = refresh_weight;
	gbfem_status st = configure_pcg(h, ctas_per_sm);
	if (st != GBFEM_OK)
	{
		const std::string msg = h->err;
		h->cgSchedule = oldSchedule;
		h->refreshWeight = oldWeight;
		configure_pcg(h, h->ctasPerSM);
		return fail(h, st, msg);
	}
	h->elemsPerBlock = elems_per_block;
	h->tuned = true;
	h->tuneVersion++;
	return GBFEM_OK;
}

gbfem_status gbfem_set_solver_params(gbfem_handle h, int32_t newton_max_iterations, double newton_epsilon,
									 double cg_tolerance, int32_t cg_max_iterations)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (newton_max_iterations < 1 || !(newton_epsilon >= 0.0) || !(cg_tolerance >= 0.0))
		return fail(h, GBFEM_INVALID_ARG, "gbfem_set_solver_params: newton_max_iterations >= 1, epsilon and tolerance >= 0");
	const bool changed = h->prm.newton_max_iterations != newton_max_iterations ||
						 h->prm.newton_epsilon != newton_epsilon || h->prm.cg_tolerance != cg_tolerance ||
						 h->prm.cg_max_iterations != cg_max_iterations;
	h->prm.newton_max_iterations = newton_max_iterations;
	h->prm.newton_epsilon = newton_epsilon;
	h->prm.cg_tolerance = cg_tolerance;
	h->prm.cg_max_iterations = cg_max_iterations;
	if (changed) h->tuneVersion++;  // a captured step graph holds the old tolerance and cap: capture again
	return GBFEM_OK;
}

gbfem_status gbfem_set_materials_device(gbfem_handle h, const double* young, const double* poisson)
{
	if (!h || !young) return GBFEM_INVALID_ARG;
	GB_CUDA(h, cudaSetDevice(h->device));
	if (h->hex())
	{
		// Stream-ordered copies of the caller's device arrays, then K and M again.
		GB_CUDA(h, cudaMemcpyAsync(h->d_young.p, young, sizeof(double) * h->E, cudaMemcpyDeviceToDevice, h->stream));
		if (poisson)
			GB_CUDA(h, cudaMemcpyAsync(h->d_poisson.p, poisson, sizeof(double) * h->E, cudaMemcpyDeviceToDevice,
									   h->stream));
		return rebuild_hex_operators(h);
	}
	if (!h->d_poisson.p)
	{
		// Each element's Poisson ratio as given (at creation or by the last call that set it), so that
		// a call that changes only E does not derive nu again from the rounded lambda V, mu V.
		GB_CUDA(h, h->d_poisson.upload(h->poissonHost.data(), h->poissonHost.size(), h->stream));
	}
	if (poisson)
		GB_CUDA(h, cudaMemcpyAsync(h->d_poisson.p, poisson, sizeof(double) * h->E, cudaMemcpyDeviceToDevice, h->stream));
	launch_set_materials(h->E, young, h->d_poisson.p, h->d_rest.p, h->mixed() ? h->d_rest32.p : nullptr, h->stream);
	h->linearReady = false;  // the stored linear system no longer matches
	GB_CUDA(h, cudaGetLastError());
	GB_CUDA(h, cudaStreamSynchronize(h->stream));
	return GBFEM_OK;
}

gbfem_status gbfem_add_external_force(gbfem_handle h, int32_t element, const double* coord, const double* force,
									   const double* stiffness, const double* damping)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (element < 0 || element >= h->E || !coord || !force)
		return fail(h, GBFEM_INVALID_ARG, "gbfem_add_external_force: bad element or null coord/force");
	const int npe = h->npe(), N = h->N;
	const int32_t* nd = &h->tets[npe * (size_t)element];
	if (!h->extPending)
	{
		h->extF.assign(h->n, 0.0);
		h->extBlocks.clear();
	}
	for (int a = 0; a < npe; ++a)
		for (int i = 0; i < 3; ++i) h->extF[3 * (size_t)nd[a] + i] += force[i] * coord[a];
	if (stiffness || damping)
		for (int a = 0; a < npe; ++a)
			for (int b = 0; b < npe; ++b)
			{
				auto it = h->extBlocks.find((int64_t)nd[a] * N + nd[b]);
				if (it == h->extBlocks.end()) it = h->extBlocks.emplace((int64_t)nd[a] * N + nd[b], std::array<double, 18>{}).first;
				const double w = coord[a] * coord[b];
				for (int k = 0; k < 9; ++k)
				{
					if (stiffness) it->second[k] += w * stiffness[k];
					if (damping) it->second[9 + k] += w * damping[k];
				}
			}
	h->extPending = true;
	return GBFEM_OK;
}

gbfem_status gbfem_adjoint_step(gbfem_handle h, double dt, const double* x, const double* v, const double* dv,
								const double* lx, const double* lv, double* lx_out, double* lv_out,
								double* grad_log_young, double* grad_poisson, uint32_t flags)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!x || !v || !dv || !lx || !lv || !lx_out || !lv_out || !(dt > 0.0))
		return fail(h, GBFEM_INVALID_ARG, "gbfem_adjoint_step: null array or dt <= 0");
	if (!h->corotational()) return fail(h, GBFEM_INVALID_ARG, "gbfem_adjoint_step: corotational elements only");
	cudaStream_t s = h->stream;
	const DevBody body = h->body();
	const int n = h->n;
	if (!h->d_mu.p)
	{
		GB_CUDA(h, h->d_mu.alloc(n));
		GB_CUDA(h, h->d_adjG.alloc(n));
		GB_CUDA(h, h->d_gx.alloc(12 * (size_t)h->E));
		GB_CUDA(h, h->d_gv.alloc(12 * (size_t)h->E));
	}
	const double alpha = h->prm.rayleigh_mass, beta = h->prm.rayleigh_stiffness;
	const double c1 = 1.0 / dt + alpha, c2 = dt + beta;
	const int maxIter = h->stepMaxIter();
	PhaseTimer tm;
	tm.init((flags & GBFEM_STEP_TIME_PHASES) != 0, s);
	tm.mark(0);
	// The step's system at (x, v), as the first Newton iteration of step_once builds it.
	int ek = 1;
	if (h->mixed())
	{
		ek = launch_element_f32(body, x, v, x, v, dt, alpha, beta, h->d_kslots32.p, h->d_rhsE32.p, h->d_counters.p, s);
		launch_assemble(body, h->d_kslots32.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
	}
	else
	{
		launch_element_fp64(body, x, v, x, v, dt, alpha, beta, h->d_kslots.p, h->d_rhsE.p, nullptr, nullptr,
							h->d_counters.p, s);
		launch_assemble(body, h->d_kslots.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
	}
	launch_adjoint_rhs(n, h->d_bc.p, lx, lv, dt, h->d_adjG.p, s);
	GB_CUDA(h, cudaGetLastError());
	h->launches += ek + 2;
	tm.mark(1);
	bool converged = true;
	if (h->persistent())
	{
		gbfem_status st = run_mixed(h, h->d_adjG.p, h->d_mu.p, maxIter, false);
		if (st != GBFEM_OK) return st;
		for (size_t k = 0; k + 1 < h->segNode.size(); ++k) converged = converged && h->h_seg[k].converged;
	}
	else
	{
		gbfem_status st = run_cg(h, h->d_adjG.p, h->d_mu.p, maxIter, false);
		if (st != GBFEM_OK) return st;
		converged = h->h_ctl->converged != 0;
	}
	tm.mark(2);
	launch_element_adjoint(body, x, v, h->d_mu.p, dv, dt, alpha, beta, h->d_gx.p, h->d_gv.p, grad_log_young,
						   grad_poisson, s, h->mixed());
	launch_adjoint_gather(body, h->d_gx.p, h->d_gv.p, lx, lv, dt, lx_out, lv_out, s);
	tm.mark(3);
	GB_CUDA(h, cudaGetLastError());
	GB_CUDA(h, cudaStreamSynchronize(s));
	h->launches += 2;
	if (tm.on)
	{
		h->stats.ms_element += tm.ms(0, 1);
		h->stats.ms_solve += tm.ms(1, 2);
		h->stats.ms_update += tm.ms(2, 3);
	}
	return converged ? GBFEM_OK : fail(h, GBFEM_CG_MAXITER, "adjoint solve did not converge");
}

}  // extern "C"

namespace {

gbfem_status ensure_adjoint_buffers(gbfem_handle h)
{
	if (h->d_mu.p) return GBFEM_OK;
	GB_CUDA(h, h->d_mu.alloc(h->n));
	GB_CUDA(h, h->d_adjG.alloc(h->n));
	GB_CUDA(h, h->d_gx.alloc(12 * (size_t)h->E));
	GB_CUDA(h, h->d_gv.alloc(12 * (size_t)h->E));
	return GBFEM_OK;
}

// The reverse of one step taken from (x, v) to (., vNext), enqueued without host synchronisation (the
// work of gbfem_adjoint_step): the step's system rebuilt at (x, v), S mu = dt lx + lv solved by the
// persistent launch (its per-segment results accumulated into d_adjAcc), the element derivatives, and
// (lx, lv) carried to the step's start in place; gradients added into glog / gnu.
gbfem_status enqueue_adjoint_step(gbfem_handle h, double dt, const double* x, const double* v, const double* vNext,
								  double* lx, double* lv, double* glog, double* gnu)
{
	cudaStream_t s = h->stream;
	const DevBody body = h->body();
	const double alpha = h->prm.rayleigh_mass, beta = h->prm.rayleigh_stiffness;
	const double c1 = 1.0 / dt + alpha, c2 = dt + beta;
	const int nseg = (int)h->segNode.size() - 1;
	launch_vec_diff(h->n, vNext, v, h->d_dvTmp.p, s);
	int k = 1;
	if (h->mixed())
	{
		k += launch_element_f32(body, x, v, x, v, dt, alpha, beta, h->d_kslots32.p, h->d_rhsE32.p, h->d_counters.p, s,
								h->elemsPerBlock);
		launch_assemble(body, h->d_kslots32.p, c1, c2, h->d_A32.p, h->d_invdiag32.p, s);
	}
	else
	{
		launch_element_fp64(body, x, v, x, v, dt, alpha, beta, h->d_kslots.p, h->d_rhsE.p, nullptr, nullptr,
							h->d_counters.p, s);
		launch_assemble(body, h->d_kslots.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
		k += 1;
	}
	launch_adjoint_rhs(h->n, h->d_bc.p, lx, lv, dt, h->d_adjG.p, s);
	gbfem_status st = enqueue_mixed(h, h->d_adjG.p, h->d_mu.p, h->stepMaxIter(), nullptr, nullptr, true);
	if (st != GBFEM_OK) return st;
	launch_step_accumulate(h->d_seg.p, nseg, &h->d_ctl.p->nonfinite, &h->d_pcgGlobal.p->err, h->d_adjAcc.p, s);
	launch_element_adjoint(body, x, v, h->d_mu.p, h->d_dvTmp.p, dt, alpha, beta, h->d_gx.p, h->d_gv.p, glog, gnu, s,
						   h->mixed());
	launch_adjoint_gather(body, h->d_gx.p, h->d_gv.p, lx, lv, dt, lx, lv, s);
	GB_CUDA(h, cudaGetLastError());
	h->launches += k + 6;
	return GBFEM_OK;
}

// Per-segment accumulators of graph-launched solves set to their start values.
gbfem_status reset_acc(gbfem_handle h, double* acc, std::vector<double>& host)
{
	const int nseg = (int)h->segNode.size() - 1;
	host.assign(4 * (size_t)nseg + 2, 0.0);
	for (int k = 0; k < nseg; ++k) host[4 * (size_t)k + 2] = 1.0;
	GB_CUDA(h, cudaMemcpyAsync(acc, host.data(), sizeof(double) * host.size(), cudaMemcpyHostToDevice, h->stream));
	return GBFEM_OK;
}

// Reads accumulated solve statistics into h->stats (and the per-segment statistics when `steps`).
void collect_acc(gbfem_handle h, const std::vector<double>& acc, bool steps)
{
	const int nseg = (int)h->segNode.size() - 1;
	double worst = 0.0;
	for (int k = 0; k < nseg; ++k)
	{
		const double* a = &acc[4 * (size_t)k];
		h->stats.cg_iterations += (int)a[0];
		h->stats.refinement_sweeps += (int)a[1];
		if (a[2] < 1.0) h->stats.cg_max_iterations_hit++;
		worst = std::max(worst, a[3]);
		if (!steps) continue;
		double* ss = &h->segStats[4 * (size_t)k];
		ss[0] += a[0];
		ss[1] += a[1];
		ss[2] = std::min(ss[2], a[2]);
		ss[3] = std::max(ss[3], a[3]);
	}
	h->stats.cg_relative_residual = worst;
}

gbfem_status rollout_checks(gbfem_handle h)
{
	if (!h->corotational()) return fail(h, GBFEM_INVALID_ARG, "rollouts: corotational elements only");
	if (!h->persistent())
		return fail(h, GBFEM_INVALID_ARG, "rollouts need the mixed form or a batch (the persistent solve)");
	if (h->prm.newton_max_iterations != 1) return fail(h, GBFEM_INVALID_ARG, "rollouts take one Newton iteration");
	if (!h->active) return fail(h, GBFEM_INACTIVE, "representation is deactivated");
	return GBFEM_OK;
}

void reset_call_stats(gbfem_handle h)
{
	std::memset(&h->stats, 0, sizeof(h->stats));
	h->launches = 0;
	for (size_t k = 0; k < h->segStats.size(); k += 4)
	{
		h->segStats[k] = h->segStats[k + 1] = h->segStats[k + 3] = 0.0;
		h->segStats[k + 2] = 1.0;
	}
}

}  // namespace

extern "C" {

gbfem_status gbfem_rollout_forward(gbfem_handle h, double dt, int32_t nsteps, int32_t checkpoint_every,
								   const double* x0, const double* v0, double* xT, double* vT)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!(dt > 0.0) || nsteps < 1 || checkpoint_every < 1 || !x0 || !v0 || !xT || !vT)
		return fail(h, GBFEM_INVALID_ARG, "gbfem_rollout_forward: dt > 0, nsteps >= 1, checkpoint_every >= 1, arrays");
	gbfem_status st = rollout_checks(h);
	if (st != GBFEM_OK) return st;
	GB_CUDA(h, cudaSetDevice(h->device));
	reset_call_stats(h);
	cudaStream_t s = h->stream;
	const size_t n = (size_t)h->n;
	const int nck = (nsteps + checkpoint_every - 1) / checkpoint_every + 1;  // + the final state
	if (h->d_ckpt.n < 2 * n * nck)
	{
		h->d_ckpt.free();
		GB_CUDA(h, h->d_ckpt.alloc(2 * n * nck));
	}
	double* ck = h->d_ckpt.p;
	GB_CUDA(h, cudaMemcpyAsync(ck, x0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(ck + n, v0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemsetAsync(h->d_counters.p, 0, 4 * sizeof(int), s));
	if (h->prm.autotune && !h->tuned)
	{
		// Tune on the first step's system (outside the graph).
		const double c1 = 1.0 / dt + h->prm.rayleigh_mass, c2 = dt + h->prm.rayleigh_stiffness;
		GB_CUDA(h, cudaMemcpyAsync(h->d_x.p, x0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		GB_CUDA(h, cudaMemcpyAsync(h->d_v.p, v0, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
		if (!h->mixed())
		{
			const DevBody body = h->body();
			launch_element_fp64(body, h->d_x.p, h->d_v.p, h->d_x.p, h->d_v.p, dt, h->prm.rayleigh_mass,
								h->prm.rayleigh_stiffness, h->d_kslots.p, h->d_rhsE.p, nullptr, nullptr, h->d_counters.p, s);
			launch_assemble(body, h->d_kslots.p, c1, c2, h->d_A.p, h->d_invdiag.p, s);
			launch_rhs_gather(body, h->d_rhsE.p, h->prm.gravity, h->prm.gravity_enabled, h->d_rhs.p, 1, s);
		}
		st = tune_mixed(h, h->d_x.p, h->d_v.p, dt, c1, c2, h->stepMaxIter());
		if (st != GBFEM_OK) return st;
	}
	if (!h->rollFwd || h->rollDt != dt || h->rollSteps != nsteps || h->rollEvery != checkpoint_every ||
		h->rollFwdVersion != h->tuneVersion)
	{
		if (h->rollFwd) cudaGraphExecDestroy(h->rollFwd);
		h->rollFwd = nullptr;
		if (h->rollBwd) cudaGraphExecDestroy(h->rollBwd);
		h->rollBwd = nullptr;
		GB_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		gbfem_status cst = GBFEM_OK;
		cudaError_t ce = cudaMemcpyAsync(h->d_x.p, ck, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
		if (ce == cudaSuccess) ce = cudaMemcpyAsync(h->d_v.p, ck + n, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
		for (int t = 0; t < nsteps && cst == GBFEM_OK && ce == cudaSuccess; ++t)
		{
			cst = enqueue_step_mixed(h, dt, false);
			const int slot = (t + 1 == nsteps) ? nck - 1 : ((t + 1) % checkpoint_every == 0 ? (t + 1) / checkpoint_every : -1);
			if (slot > 0 && cst == GBFEM_OK)
			{
				ce = cudaMemcpyAsync(ck + 2 * n * slot, h->d_x.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
				if (ce == cudaSuccess)
					ce = cudaMemcpyAsync(ck + 2 * n * slot + n, h->d_v.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
			}
		}
		cudaGraph_t graph = nullptr;
		const cudaError_t ee = cudaStreamEndCapture(s, &graph);
		if (cst != GBFEM_OK || ce != cudaSuccess || ee != cudaSuccess)
		{
			if (graph) cudaGraphDestroy(graph);
			if (cst != GBFEM_OK) return cst;
			GB_CUDA(h, ce != cudaSuccess ? ce : ee);
		}
		const cudaError_t ie = cudaGraphInstantiate(&h->rollFwd, graph, 0);
		cudaGraphDestroy(graph);
		GB_CUDA(h, ie);
		h->rollDt = dt;
		h->rollSteps = nsteps;
		h->rollEvery = checkpoint_every;
		h->rollFwdVersion = h->tuneVersion;
	}
	std::vector<double> acc;
	st = reset_acc(h, h->d_acc.p, acc);
	if (st != GBFEM_OK) return st;
	GB_CUDA(h, cudaMemsetAsync(h->d_pcgGlobal.p, 0, sizeof(PcgGlobal), s));
	GB_CUDA(h, cudaGraphLaunch(h->rollFwd, s));
	h->launches += nsteps * h->graphKernels;
	GB_CUDA(h, cudaMemcpyAsync(xT, h->d_x.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(vT, h->d_v.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(acc.data(), h->d_acc.p, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, s));
	int counters[4] = {0, 0, 0, 0};
	GB_CUDA(h, cudaMemcpyAsync(counters, h->d_counters.p, sizeof(counters), cudaMemcpyDeviceToHost, s));
	GB_CUDA(h, cudaStreamSynchronize(s));
	GB_CUDA(h, cudaGetLastError());
	collect_acc(h, acc, true);
	h->stats.steps = nsteps;
	h->stats.singular_g = counters[0];
	h->stats.polar_fallbacks = counters[1];
	h->stats.kernel_launches = h->launches;
	h->stats.active = 1;
	h->systemReady = true;
	h->lastDt = dt;
	const int nseg = (int)h->segNode.size() - 1;
	if (acc[4 * (size_t)nseg + 1] != 0.0) return fail(h, GBFEM_CUDA_ERROR, "persistent CG: grid barrier timed out");
	if (acc[4 * (size_t)nseg] != 0.0)
	{
		h->active = false;
		h->stats.active = 0;
		return fail(h, GBFEM_NONFINITE, "state is not finite during the rollout; representation deactivated");
	}
	if (h->stats.cg_max_iterations_hit > 0) return fail(h, GBFEM_CG_MAXITER, "CG reached its maximum number of iterations");
	return GBFEM_OK;
}

gbfem_status gbfem_rollout_backward(gbfem_handle h, const double* lxT, const double* lvT, double* lx0, double* lv0,
									double* grad_log_young, double* grad_poisson)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!lxT || !lvT || !lx0 || !lv0) return fail(h, GBFEM_INVALID_ARG, "gbfem_rollout_backward: null array");
	gbfem_status st = rollout_checks(h);
	if (st != GBFEM_OK) return st;
	if (!h->rollFwd || h->rollFwdVersion != h->tuneVersion)
		return fail(h, GBFEM_INVALID_ARG, "gbfem_rollout_backward: no forward rollout to reverse");
	GB_CUDA(h, cudaSetDevice(h->device));
	reset_call_stats(h);
	cudaStream_t s = h->stream;
	const size_t n = (size_t)h->n, E = (size_t)h->E;
	const int nsteps = h->rollSteps, every = h->rollEvery;
	const double dt = h->rollDt;
	const int nck = (nsteps + every - 1) / every + 1;
	st = ensure_adjoint_buffers(h);
	if (st != GBFEM_OK) return st;
	if (!h->d_segX.p)
	{
		const int nseg = (int)h->segNode.size() - 1;
		GB_CUDA(h, h->d_rollL.alloc(2 * n));
		GB_CUDA(h, h->d_rollG.alloc(2 * E));
		GB_CUDA(h, h->d_dvTmp.alloc(n));
		GB_CUDA(h, h->d_adjAcc.alloc(4 * (size_t)nseg + 2));
	}
	if (h->d_segX.n < 2 * n * (size_t)(every + 1))
	{
		h->d_segX.free();
		GB_CUDA(h, h->d_segX.alloc(2 * n * (size_t)(every + 1)));
	}
	double* ck = h->d_ckpt.p;
	double* sx = h->d_segX.p;
	double* lx = h->d_rollL.p;
	double* lv = lx + n;
	double* gl = h->d_rollG.p;
	double* gn = gl + E;
	GB_CUDA(h, cudaMemcpyAsync(lx, lxT, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(lv, lvT, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemsetAsync(h->d_counters.p, 0, 4 * sizeof(int), s));
	if (!h->rollBwd || h->rollBwdVersion != h->tuneVersion)
	{
		if (h->rollBwd) cudaGraphExecDestroy(h->rollBwd);
		h->rollBwd = nullptr;
		GB_CUDA(h, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
		gbfem_status cst = GBFEM_OK;
		cudaError_t ce = cudaMemsetAsync(gl, 0, sizeof(double) * 2 * E, s);
		auto copy = [&](double* dst, const double* src) {
			if (ce == cudaSuccess) ce = cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToDevice, s);
		};
		const int nsegs = nck - 1;
		// With a checkpoint after every step (every == 1) the forward kept every state (2n doubles a
		// step): the reverse sweep re-runs no step.
		for (int t = nsteps - 1; every == 1 && t >= 0 && cst == GBFEM_OK && ce == cudaSuccess; --t)
			cst = enqueue_adjoint_step(h, dt, ck + 2 * n * t, ck + 2 * n * t + n, ck + 2 * n * (t + 1) + n, lx, lv, gl, gn);
		for (int sg = nsegs - 1; every > 1 && sg >= 0 && cst == GBFEM_OK && ce == cudaSuccess; --sg)
		{
			const int len = std::min(every, nsteps - sg * every);
			copy(h->d_x.p, ck + 2 * n * sg);
			copy(h->d_v.p, ck + 2 * n * sg + n);
			copy(sx, h->d_x.p);
			copy(sx + n, h->d_v.p);
			for (int j = 0; j < len && cst == GBFEM_OK && ce == cudaSuccess; ++j)
			{
				cst = enqueue_step_mixed(h, dt, false);
				copy(sx + 2 * n * (j + 1), h->d_x.p);
				copy(sx + 2 * n * (j + 1) + n, h->d_v.p);
			}
			for (int j = len - 1; j >= 0 && cst == GBFEM_OK && ce == cudaSuccess; --j)
				cst = enqueue_adjoint_step(h, dt, sx + 2 * n * j, sx + 2 * n * j + n, sx + 2 * n * (j + 1) + n, lx, lv, gl,
										   gn);
		}
		copy(h->d_x.p, ck + 2 * n * (nck - 1));  // the handle keeps the forward's final state
		copy(h->d_v.p, ck + 2 * n * (nck - 1) + n);
		cudaGraph_t graph = nullptr;
		const cudaError_t ee = cudaStreamEndCapture(s, &graph);
		if (cst != GBFEM_OK || ce != cudaSuccess || ee != cudaSuccess)
		{
			if (graph) cudaGraphDestroy(graph);
			if (cst != GBFEM_OK) return cst;
			GB_CUDA(h, ce != cudaSuccess ? ce : ee);
		}
		const cudaError_t ie = cudaGraphInstantiate(&h->rollBwd, graph, 0);
		cudaGraphDestroy(graph);
		GB_CUDA(h, ie);
		h->rollBwdVersion = h->tuneVersion;
	}
	std::vector<double> acc, adj;
	st = reset_acc(h, h->d_acc.p, acc);
	if (st == GBFEM_OK) st = reset_acc(h, h->d_adjAcc.p, adj);
	if (st != GBFEM_OK) return st;
	GB_CUDA(h, cudaMemsetAsync(h->d_pcgGlobal.p, 0, sizeof(PcgGlobal), s));
	GB_CUDA(h, cudaGraphLaunch(h->rollBwd, s));
	GB_CUDA(h, cudaMemcpyAsync(lx0, lx, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(lv0, lv, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
	if (grad_log_young) GB_CUDA(h, cudaMemcpyAsync(grad_log_young, gl, sizeof(double) * E, cudaMemcpyDeviceToDevice, s));
	if (grad_poisson) GB_CUDA(h, cudaMemcpyAsync(grad_poisson, gn, sizeof(double) * E, cudaMemcpyDeviceToDevice, s));
	GB_CUDA(h, cudaMemcpyAsync(acc.data(), h->d_acc.p, sizeof(double) * acc.size(), cudaMemcpyDeviceToHost, s));
	GB_CUDA(h, cudaMemcpyAsync(adj.data(), h->d_adjAcc.p, sizeof(double) * adj.size(), cudaMemcpyDeviceToHost, s));
	GB_CUDA(h, cudaStreamSynchronize(s));
	GB_CUDA(h, cudaGetLastError());
	collect_acc(h, acc, false);
	const int fwdHit = h->stats.cg_max_iterations_hit;
	collect_acc(h, adj, false);
	h->stats.steps = nsteps;
	h->stats.kernel_launches = h->launches;
	h->stats.active = 1;
	const int nseg = (int)h->segNode.size() - 1;
	if (acc[4 * (size_t)nseg + 1] != 0.0 || adj[4 * (size_t)nseg + 1] != 0.0)
		return fail(h, GBFEM_CUDA_ERROR, "persistent CG: grid barrier timed out");
	if (acc[4 * (size_t)nseg] != 0.0) return fail(h, GBFEM_NONFINITE, "a re-run state is not finite");
	if (h->stats.cg_max_iterations_hit > fwdHit || fwdHit > 0)
		return fail(h, GBFEM_CG_MAXITER, "a solve of the reverse sweep did not converge");
	return GBFEM_OK;
}

gbfem_status gbfem_batch_info(gbfem_handle h, int32_t* count, int32_t* node_offsets, int32_t* tet_offsets,
							  int64_t* nnz_per_mesh)
{
	if (!h) return GBFEM_INVALID_ARG;
	const int nseg = (int)h->segNode.size() - 1;
	if (count) *count = nseg;
	if (node_offsets) std::copy(h->segNode.begin(), h->segNode.end(), node_offsets);
	if (tet_offsets) std::copy(h->segTet.begin(), h->segTet.end(), tet_offsets);
	if (nnz_per_mesh)
		for (int k = 0; k < nseg; ++k)
			nnz_per_mesh[k] = 9LL * (h->adjPtr[h->segNode[k + 1]] - h->adjPtr[h->segNode[k]]);
	return GBFEM_OK;
}

gbfem_status gbfem_batch_segment_stats(gbfem_handle h, int32_t* iterations, int32_t* refreshes, int32_t* converged,
									   double* relative_residual)
{
	if (!h) return GBFEM_INVALID_ARG;
	const size_t nseg = h->segNode.size() - 1;
	for (size_t k = 0; k < nseg; ++k)
	{
		if (iterations) iterations[k] = (int32_t)h->segStats[4 * k];
		if (refreshes) refreshes[k] = (int32_t)h->segStats[4 * k + 1];
		if (converged) converged[k] = (int32_t)h->segStats[4 * k + 2];
		if (relative_residual) relative_residual[k] = h->segStats[4 * k + 3];
	}
	return GBFEM_OK;
}

gbfem_status gbfem_destroy(gbfem_handle h)
{
	if (!h) return GBFEM_INVALID_ARG;
	cudaSetDevice(h->device);
	if (h->stream) cudaStreamSynchronize(h->stream);
	h->release();
	delete h;
	return GBFEM_OK;
}

gbfem_status gbfem_step(gbfem_handle h, double dt, int32_t nsteps, uint32_t flags)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!(dt > 0.0) || nsteps < 0) return fail(h, GBFEM_INVALID_ARG, "dt must be > 0 and nsteps >= 0");
	std::memset(&h->stats, 0, sizeof(h->stats));
	h->launches = 0;
	for (size_t k = 0; k < h->segStats.size(); k += 4)
	{
		h->segStats[k] = h->segStats[k + 1] = h->segStats[k + 3] = 0.0;
		h->segStats[k + 2] = 1.0;
	}
	if (!h->active)
	{
		h->stats.active = 0;
		return fail(h, GBFEM_INACTIVE, "representation is deactivated");
	}
	GB_CUDA(h, cudaSetDevice(h->device));
	GB_CUDA(h, cudaMemsetAsync(h->d_counters.p, 0, 4 * sizeof(int), h->stream));
	gbfem_status result = GBFEM_OK;
	int sidx = 0;
	// Pending external forces apply to the first step of this call only (the reference clears them
	// after each update, DeformableRepresentation::afterUpdate).
	h->extActive = h->extPending && nsteps > 0;
	const bool needPlainStep = (h->prm.autotune && !h->tuned) || (h->constantSystem() && !h->systemCurrent(dt)) ||
							   h->extActive;
	auto end_external = [&]() {
		if (!h->extActive) return;
		h->extActive = false;
		h->extPending = false;
		h->extBlocks.clear();
		std::fill(h->extF.begin(), h->extF.end(), 0.0);
		if (h->constantSystem()) h->linearReady = false;  // the stored system holds this step's K_ext, D_ext
	};
	if ((flags & GBFEM_STEP_GRAPH) && needPlainStep && nsteps > 0)
	{
		result = step_once(h, dt, flags & ~GBFEM_STEP_GRAPH);  // the first step tunes, outside any graph
		end_external();
		sidx = 1;
		const bool fatal = result == GBFEM_NONFINITE || result == GBFEM_CUDA_ERROR || result == GBFEM_OUT_OF_MEMORY ||
						   result == GBFEM_INVALID_ARG;
		if (!fatal && sidx < nsteps && h->constantSystem() && !h->systemCurrent(dt))
		{
			result = step_once(h, dt, flags & ~GBFEM_STEP_GRAPH);  // rebuild the stored system without K_ext
			sidx = 2;
		}
	}
	if ((flags & GBFEM_STEP_GRAPH) && sidx < nsteps &&
		!(result == GBFEM_NONFINITE || result == GBFEM_CUDA_ERROR || result == GBFEM_OUT_OF_MEMORY))
	{
		gbfem_status st = step_graph(h, dt, nsteps - sidx, flags);
		if (st != GBFEM_OK) result = st;
		sidx = nsteps;
	}
	for (; sidx < nsteps; ++sidx)
	{
		gbfem_status st = step_once(h, dt, flags);
		end_external();
		if (st == GBFEM_NONFINITE || st == GBFEM_CUDA_ERROR || st == GBFEM_OUT_OF_MEMORY || st == GBFEM_INVALID_ARG)
		{
			result = st;
			break;
		}
	}
	int counters[4] = {0, 0, 0, 0};
	cudaMemcpy(counters, h->d_counters.p, sizeof(counters), cudaMemcpyDeviceToHost);
	h->stats.singular_g = counters[0];
	h->stats.polar_fallbacks = counters[1];
	h->stats.active = h->active ? 1 : 0;
	h->stats.kernel_launches = h->launches;
	if (result == GBFEM_OK && h->stats.cg_max_iterations_hit > 0)
	{
		h->err = "CG reached its maximum number of iterations";
		result = GBFEM_CG_MAXITER;
	}
	return result;
}

gbfem_status gbfem_get_stats(gbfem_handle h, gbfem_stats* out)
{
	if (!h || !out) return GBFEM_INVALID_ARG;
	*out = h->stats;
	return GBFEM_OK;
}

gbfem_status gbfem_get_state(gbfem_handle h, double* x, double* v)
{
	if (!h) return GBFEM_INVALID_ARG;
	GB_CUDA(h, cudaSetDevice(h->device));
	if (x) GB_CUDA(h, cudaMemcpyAsync(x, h->d_x.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
	if (v) GB_CUDA(h, cudaMemcpyAsync(v, h->d_v.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
	GB_CUDA(h, cudaStreamSynchronize(h->stream));
	return GBFEM_OK;
}

gbfem_status gbfem_set_state(gbfem_handle h, const double* x, const double* v)
{
	if (!h) return GBFEM_INVALID_ARG;
	GB_CUDA(h, cudaSetDevice(h->device));
	if (x) GB_CUDA(h, cudaMemcpyAsync(h->d_x.p, x, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->stream));
	if (v) GB_CUDA(h, cudaMemcpyAsync(h->d_v.p, v, sizeof(double) * h->n, cudaMemcpyHostToDevice, h->stream));
	GB_CUDA(h, cudaStreamSynchronize(h->stream));
	return GBFEM_OK;
}

gbfem_status gbfem_set_velocities(gbfem_handle h, int32_t count, const int32_t* dofs, const double* values)
{
	if (!h || count < 0 || (count > 0 && (!dofs || !values))) return GBFEM_INVALID_ARG;
	for (int32_t i = 0; i < count; ++i)
		if (dofs[i] < 0 || dofs[i] >= h->n) return fail(h, GBFEM_INVALID_ARG, "dof out of range");
	if (count == 0) return GBFEM_OK;
	GB_CUDA(h, cudaSetDevice(h->device));
	if (h->d_idx.n < (size_t)count)
	{
		GB_CUDA(h, h->d_idx.alloc(count));
		GB_CUDA(h, h->d_vals.alloc(count));
	}
	GB_CUDA(h, cudaMemcpyAsync(h->d_idx.p, dofs, sizeof(int) * count, cudaMemcpyHostToDevice, h->stream));
	GB_CUDA(h, cudaMemcpyAsync(h->d_vals.p, values, sizeof(double) * count, cudaMemcpyHostToDevice, h->stream));
	launch_scatter_values(count, h->d_idx.p, h->d_vals.p, h->d_v.p, h->stream);
	GB_CUDA(h, cudaStreamSynchronize(h->stream));
	GB_CUDA(h, cudaGetLastError());
	return GBFEM_OK;
}

gbfem_status gbfem_set_velocities_device(gbfem_handle h, int32_t count, const int32_t* dofs_dev,
										 const double* values_dev)
{
	if (!h || count < 0 || (count > 0 && (!dofs_dev || !values_dev))) return GBFEM_INVALID_ARG;
	if (count == 0) return GBFEM_OK;
	GB_CUDA(h, cudaSetDevice(h->device));
	launch_scatter_values(count, dofs_dev, values_dev, h->d_v.p, h->stream);
	GB_CUDA(h, cudaGetLastError());
	return GBFEM_OK;
}

gbfem_status gbfem_device_state(gbfem_handle h, double** x, double** v)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (x) *x = h->d_x.p;
	if (v) *v = h->d_v.p;
	return GBFEM_OK;
}

gbfem_status gbfem_stream(gbfem_handle h, void** stream)
{
	if (!h || !stream) return GBFEM_INVALID_ARG;
	*stream = (void*)h->stream;
	return GBFEM_OK;
}

gbfem_status gbfem_reactivate(gbfem_handle h)
{
	if (!h) return GBFEM_INVALID_ARG;
	h->active = true;
	return GBFEM_OK;
}

gbfem_status gbfem_get_sizes(gbfem_handle h, int64_t* num_dofs, int64_t* nnz)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (num_dofs) *num_dofs = h->n;
	if (nnz) *nnz = h->nnz;
	return GBFEM_OK;
}

gbfem_status gbfem_get_pattern(gbfem_handle h, int32_t* colptr, int32_t* rowidx)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (colptr)
	{
		colptr[0] = 0;
		for (int J = 0; J < h->N; ++J)
		{
			int deg = h->adjPtr[J + 1] - h->adjPtr[J];
			for (int j = 0; j < 3; ++j) colptr[3 * J + j + 1] = (int32_t)(9LL * h->adjPtr[J] + 3LL * (j + 1) * deg);
		}
	}
	if (rowidx)
	{
		int64_t k = 0;
		for (int J = 0; J < h->N; ++J)
			for (int j = 0; j < 3; ++j)
				for (int t = h->adjPtr[J]; t < h->adjPtr[J + 1]; ++t)
					for (int i = 0; i < 3; ++i) rowidx[k++] = 3 * h->adj[t] + i;
	}
	return GBFEM_OK;
}

gbfem_status gbfem_get_scatter(gbfem_handle h, int32_t* map)
{
	if (!h || !map) return GBFEM_INVALID_ARG;
	const int npe = h->npe(), D = 3 * npe;
	for (int e = 0; e < h->E; ++e)
	{
		const int* nd = &h->tets[npe * (size_t)e];
		for (int a = 0; a < npe; ++a)
			for (int b = 0; b < npe; ++b)
				for (int j = 0; j < 3; ++j)
				{
					int64_t first = h->cscSlot(3 * nd[a], 3 * nd[b] + j);
					for (int i = 0; i < 3; ++i)
						map[(size_t)e * D * D + (3 * a + i) * D + 3 * b + j] = (int32_t)(first + i);
				}
	}
	return GBFEM_OK;
}

gbfem_status gbfem_get_system(gbfem_handle h, double* S, double* rhs, double* f)
{
	if (!h) return GBFEM_INVALID_ARG;
	if (!h->haveSystem) return fail(h, GBFEM_INVALID_ARG, "no system kept: step with GBFEM_STEP_KEEP_SYSTEM first");
	GB_CUDA(h, cudaSetDevice(h->device));
	if (S) GB_CUDA(h, cudaMemcpyAsync(S, h->d_S.p, sizeof(double) * h->nnz, cudaMemcpyDeviceToHost, h->stream));
	if (rhs) GB_CUDA(h, cudaMemcpyAsync(rhs, h->d_rhs.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
	if (f) GB_CUDA(h, cudaMemcpyAsync(f, h->d_f.p, sizeof(double) * h->n, cudaMemcpyDeviceToHost, h->stream));
	GB_CUDA(h, cudaStreamSynchronize(h->stream));
	return GBFEM_OK;
}

gbfem_status gbfem_last_error(gbfem_handle h, char* buf, size_t len)
{
	if (!buf || len == 0) return GBFEM_INVALID_ARG;
	const std::string& s = h ? h->err : g_lastCreateError;
	std::snprintf(buf, len, "%s", s.c_str());
	return GBFEM_OK;
}

gbfem_status gbfem_barrier_selftest(int32_t phases, int32_t stall, int64_t timeout_ns, int32_t* phases_passed,
									int64_t* max_wait_ns)
{
	if (phases < 1 || phases > 1000000 || timeout_ns < 1000 || timeout_ns > 2000000000LL)
	{
		set_global_error("gbfem_barrier_selftest: phases must be in [1, 1e6] and timeout_ns in [1000, 2e9]");
		return GBFEM_INVALID_ARG;
	}
	auto cuda_fail = [](const char* what, cudaError_t e) {
		set_global_error(std::string("gbfem_barrier_selftest: ") + what + ": " + cudaGetErrorString(e));
		return GBFEM_CUDA_ERROR;
	};
	int dev = 0, sms = 0, coop = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
	if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
	if (e != cudaSuccess) return cuda_fail("device query", e);
	if (!coop || sms < 2)
	{
		set_global_error("gbfem_barrier_selftest: the device has no cooperative launch or fewer than 2 SMs");
		return GBFEM_CUDA_ERROR;
	}
	const int G = sms;  // one 32-thread block per SM: co-resident, as the cooperative launch checks
	DevBuf<PcgGlobal> g;
	DevBuf<long long> out;
	auto release = [&]() {
		g.free();
		out.free();
	};
	e = g.alloc(1);
	if (e == cudaSuccess) e = out.alloc(2 * (size_t)G);
	if (e != cudaSuccess)
	{
		release();
		return cuda_fail("cudaMalloc", e);
	}
	cudaStream_t st = nullptr;
	e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
	if (e != cudaSuccess)
	{
		release();
		return cuda_fail("cudaStreamCreate", e);
	}
	e = cudaMemsetAsync(g.p, 0, sizeof(PcgGlobal), st);
	if (e == cudaSuccess) e = cudaMemsetAsync(out.p, 0, sizeof(long long) * 2 * G, st);
	if (e == cudaSuccess)
	{
		cudaLaunchConfig_t cfg = {};
		cfg.gridDim = dim3(G);
		cfg.blockDim = dim3(32);
		cfg.stream = st;
		cudaLaunchAttribute attr[1];
		attr[0].id = cudaLaunchAttributeCooperative;
		attr[0].val.cooperative = 1;
		cfg.attrs = attr;
		cfg.numAttrs = 1;
		e = cudaLaunchKernelEx(&cfg, k_barrier_selftest, g.p, (int)phases, (int)(stall != 0), (long long)timeout_ns,
							   out.p);
	}
	std::vector<long long> hout(2 * (size_t)G, 0);
	PcgGlobal hg = {};
	if (e == cudaSuccess) e = cudaMemcpyAsync(hout.data(), out.p, sizeof(long long) * 2 * G, cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&hg, g.p, sizeof(PcgGlobal), cudaMemcpyDeviceToHost, st);
	if (e == cudaSuccess) e = cudaStreamSynchronize(st);
	cudaStreamDestroy(st);
	release();
	if (e != cudaSuccess) return cuda_fail("launch", e);
	long long minPassed = phases, maxWait = 0;
	for (int b = 0; b < G; ++b)
	{
		minPassed = std::min(minPassed, hout[2 * b]);
		maxWait = std::max(maxWait, hout[2 * b + 1]);
	}
	if (phases_passed) *phases_passed = (int32_t)minPassed;
	if (max_wait_ns) *max_wait_ns = maxWait;
	if (hg.err || minPassed < phases)
	{
		set_global_error("gbfem_barrier_selftest: a grid-barrier wait ran out after " + std::to_string(timeout_ns) +
						 " ns; fewest barriers passed by a block: " + std::to_string(minPassed));
		return GBFEM_CUDA_ERROR;
	}
	return GBFEM_OK;
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// LinearSparseSolveAndInverseCG on a caller matrix.
// ------------------------------------------------------------------------------------------
struct gbfem_cg_s
{
	int device = 0, n = 0;
	double tol = DBL_EPSILON;
	int maxIter = 0;
	cudaStream_t stream = nullptr;
	DevBuf<int> rowptr, col;
	DevBuf<double> val, invdiag, b, x, r, p, q, part;
	DevBuf<CgCtl> ctl;
	CgCtl* h_ctl = nullptr;
	void release()
	{
		rowptr.free();
		col.free();
		for (auto* d : {&val, &invdiag, &b, &x, &r, &p, &q, &part}) d->free();
		ctl.free();
		if (h_ctl) cudaFreeHost(h_ctl);
		h_ctl = nullptr;
		if (stream) cudaStreamDestroy(stream);
		stream = nullptr;
	}
};

extern "C" {

gbfem_status gbfem_cg_create(int32_t n, const int32_t* colptr, const int32_t* rowidx, const double* values,
							 int32_t device, gbfem_cg* out)
{
	if (!out || n <= 0 || !colptr || !rowidx || !values) return fail(nullptr, GBFEM_INVALID_ARG, "bad CG matrix");
	*out = nullptr;
	if (colptr[0] != 0) return fail(nullptr, GBFEM_INVALID_ARG, "colptr[0] must be 0");
	for (int c = 0; c < n; ++c)
		if (colptr[c + 1] < colptr[c]) return fail(nullptr, GBFEM_INVALID_ARG, "colptr not monotone");
	for (int64_t k = 0; k < colptr[n]; ++k)
		if (rowidx[k] < 0 || rowidx[k] >= n) return fail(nullptr, GBFEM_INVALID_ARG, "row index out of range");
	// Symmetric CSR from the lower triangle (row >= col) of the CSC matrix.
	std::vector<int> cnt(n + 1, 0);
	std::vector<double> invd(n, 1.0);
	for (int c = 0; c < n; ++c)
		for (int k = colptr[c]; k < colptr[c + 1]; ++k)
		{
			int r = rowidx[k];
			if (r < c) continue;
			cnt[r + 1]++;
			if (r != c) cnt[c + 1]++;
			if (r == c && values[k] != 0.0) invd[r] = 1.0 / values[k];
		}
	for (int i = 0; i < n; ++i) cnt[i + 1] += cnt[i];
	std::vector<std::pair<int, double>> ent(cnt[n]);
	{
		std::vector<int> fill(cnt.begin(), cnt.end() - 1);
		for (int c = 0; c < n; ++c)
			for (int k = colptr[c]; k < colptr[c + 1]; ++k)
			{
				int r = rowidx[k];
				if (r < c) continue;
				ent[fill[r]++] = {c, values[k]};
				if (r != c) ent[fill[c]++] = {r, values[k]};
			}
	}
	std::vector<int> colv(ent.size());
	std::vector<double> valv(ent.size());
	for (int i = 0; i < n; ++i)
	{
		std::sort(ent.begin() + cnt[i], ent.begin() + cnt[i + 1],
				  [](const std::pair<int, double>& a, const std::pair<int, double>& b) { return a.first < b.first; });
		for (int k = cnt[i]; k < cnt[i + 1]; ++k)
		{
			colv[k] = ent[k].first;
			valv[k] = ent[k].second;
		}
	}
	auto* g = new gbfem_cg_s();
	g->device = device;
	g->n = n;
	auto bad = [&](cudaError_t e) {
		std::string msg = std::string("CUDA: ") + cudaGetErrorString(e);
		g->release();
		delete g;
		return fail(nullptr, e == cudaErrorMemoryAllocation ? GBFEM_OUT_OF_MEMORY : GBFEM_CUDA_ERROR, msg);
	};
	cudaError_t e = cudaSetDevice(device);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = g->rowptr.upload(cnt.data(), n + 1, g->stream);
	if (e == cudaSuccess) e = g->col.upload(colv.data(), colv.size(), g->stream);
	if (e == cudaSuccess) e = g->val.upload(valv.data(), valv.size(), g->stream);
	if (e == cudaSuccess) e = g->invdiag.upload(invd.data(), n, g->stream);
	for (auto* d : {&g->b, &g->x, &g->r, &g->p, &g->q})
		if (e == cudaSuccess) e = d->alloc(n);
	int grid = std::max(1, std::min((n + 255) / 256, 152 * 8));
	if (e == cudaSuccess) e = g->part.alloc(partial_slots(grid));
	if (e == cudaSuccess) e = g->ctl.alloc(1);
	if (e == cudaSuccess) e = cudaMemsetAsync(g->ctl.p, 0, sizeof(CgCtl), g->stream);
	if (e == cudaSuccess) e = cudaMallocHost(&g->h_ctl, sizeof(CgCtl));
	if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
	if (e != cudaSuccess) return bad(e);
	*out = g;
	return GBFEM_OK;
}

gbfem_status gbfem_cg_set_tolerance(gbfem_cg cg, double tolerance)
{
	if (!cg || !(tolerance >= 0.0)) return GBFEM_INVALID_ARG;
	cg->tol = tolerance;
	return GBFEM_OK;
}

gbfem_status gbfem_cg_set_max_iterations(gbfem_cg cg, int32_t max_iterations)
{
	if (!cg) return GBFEM_INVALID_ARG;
	cg->maxIter = max_iterations;
	return GBFEM_OK;
}

gbfem_status gbfem_cg_solve(gbfem_cg cg, const double* b, double* x, int32_t* iterations, double* relative_residual)
{
	if (!cg || !b || !x) return GBFEM_INVALID_ARG;
	auto cuda = [](cudaError_t e) { return e == cudaSuccess; };
	if (!cuda(cudaSetDevice(cg->device))) return GBFEM_CUDA_ERROR;
	Launch L;
	L.stream = cg->stream;
	L.vecGrid = std::max(1, std::min((cg->n + 255) / 256, 152 * 8));
	const int maxIter = cg->maxIter > 0 ? cg->maxIter : 2 * cg->n;
	if (!cuda(cudaMemcpyAsync(cg->b.p, b, sizeof(double) * cg->n, cudaMemcpyHostToDevice, cg->stream)))
		return GBFEM_CUDA_ERROR;
	MatCsr A{cg->n, cg->rowptr.p, cg->col.p, cg->val.p};
	launch_cg_init(cg->n, cg->b.p, cg->invdiag.p, cg->x.p, cg->r.p, cg->p.p, cg->ctl.p, cg->part.p, cg->tol, maxIter, L);
	long long launched = 0;
	int chunk = 4;
	for (;;)
	{
		for (int k = 0; k < chunk; ++k)
		{
			launch_cg_spmv_csr(A, cg->p.p, cg->q.p, cg->ctl.p, cg->part.p, L);
			launch_cg_update(cg->n, cg->invdiag.p, cg->p.p, cg->q.p, cg->x.p, cg->r.p, cg->ctl.p, cg->part.p, L);
			launch_cg_pupdate(cg->n, cg->invdiag.p, cg->r.p, cg->p.p, cg->ctl.p, L);
		}
		launched += chunk;
		if (!cuda(cudaMemcpyAsync(cg->h_ctl, cg->ctl.p, sizeof(CgCtl), cudaMemcpyDeviceToHost, cg->stream)) ||
			!cuda(cudaStreamSynchronize(cg->stream)))
			return GBFEM_CUDA_ERROR;
		if (cg->h_ctl->done) break;
		if (launched > (long long)maxIter + 64) return GBFEM_CUDA_ERROR;
		chunk = std::min(chunk * 2, 32);
	}
	if (!cuda(cudaMemcpyAsync(x, cg->x.p, sizeof(double) * cg->n, cudaMemcpyDeviceToHost, cg->stream)) ||
		!cuda(cudaStreamSynchronize(cg->stream)) || !cuda(cudaGetLastError()))
		return GBFEM_CUDA_ERROR;
	if (iterations) *iterations = cg->h_ctl->iter;
	if (relative_residual) *relative_residual = cg->h_ctl->bb > 0 ? std::sqrt(cg->h_ctl->rr / cg->h_ctl->bb) : 0.0;
	return cg->h_ctl->converged ? GBFEM_OK : GBFEM_CG_MAXITER;
}

gbfem_status gbfem_cg_destroy(gbfem_cg cg)
{
	if (!cg) return GBFEM_INVALID_ARG;
	cudaSetDevice(cg->device);
	cg->release();
	delete cg;
	return GBFEM_OK;
}

}  // extern "C"
