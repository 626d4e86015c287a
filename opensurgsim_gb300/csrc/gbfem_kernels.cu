// gbfem_kernels.cu -- sm_103a kernels of the corotational-tetrahedron implicit-Euler step.
//
// Element kernels (one element per thread; the math is in gbfem_element.cuh), deterministic
// gather assembly into a symmetric SELL-32 block matrix built from the lower triangle (Eigen's
// ConjugateGradient<..., Lower> reads only that triangle), the per-node right-hand-side gather,
// the FP64 Jacobi-PCG. The mixed-precision solve is the persistent kernel of gbfem_pcg.cu.

#include <cfloat>
#include <cstdint>

#include "gbfem_element.cuh"
#include "gbfem_internal.h"

namespace gbfem {

namespace {

constexpr int kVecThreads = 256;
constexpr int kElemThreads = 64;

// ------------------------------------------------------------------------------------------
// Element kernels
// ------------------------------------------------------------------------------------------
template <bool kDebug, bool kLinear>
__global__ void __launch_bounds__(kElemThreads) k_element_fp64(DevBody b, const double* __restrict__ xn,
																const double* __restrict__ vn,
																const double* __restrict__ xt,
																const double* __restrict__ vt, double dt, double alpha,
																double beta, double* __restrict__ kslots,
																double* __restrict__ rhsE, double* __restrict__ kfull,
																double* __restrict__ fE, int* counters)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= b.E) return;
	const int E = b.E;
	elem::ElemIn in;
	elem::gather(b, e, xn, vn, xt, vt, dt, alpha, beta, in);
	double g[4][3];
#pragma unroll
	for (int a = 0; a < 4; ++a)
#pragma unroll
		for (int k = 0; k < 3; ++k) g[a][k] = b.rest[(3 * a + k) * E + e];
	const double lamV = b.rest[13 * E + e], muV = b.rest[14 * E + e], cm = b.rest[15 * E + e];
	const int fl = elem::compute<double, kDebug, elem::ElemIn, kLinear>(
		in, g, lamV, muV, cm, kslots ? kslots + (size_t)e * (kSlots * 9) : nullptr, 1, rhsE + (size_t)e * 12, 1,
		kDebug ? kfull + (size_t)e * 144 : nullptr, kDebug ? fE + (size_t)e * 12 : nullptr);
	if (fl & 1) atomicAdd(&counters[1], 1);
	if (fl & 2) atomicAdd(&counters[0], 1);
}

// Node pass of the FP32 corotational element kernel: its per-dof inputs formed once per node rather
// than once per incident element (~24 elements a node), in the only FP64 arithmetic of the FP32
// element update: x as an unevaluated float pair (hi = x rounded, lo = x - hi rounded), v, and,
// past the first Newton iteration, x_n - x_t and v_n - v_t.
__global__ void k_node_prep(int n, const double* __restrict__ xn, const double* __restrict__ vn,
							const double* __restrict__ xt, const double* __restrict__ vt, bool start,
							float2* __restrict__ X, float* __restrict__ V, float* __restrict__ Dx,
							float* __restrict__ Dv)
{
	const int d = blockIdx.x * blockDim.x + threadIdx.x;
	if (d >= n) return;
	const double x = xn[d], v = vn[d];
	const float hi = float(x);
	X[d] = make_float2(hi, float(x - double(hi)));
	V[d] = float(v);
	if (!start)
	{
		Dx[d] = float(x - xt[d]);
		Dv[d] = float(v - vt[d]);
	}
}

// FP32 element kernel of the mixed form, kT elements per block (a tuning choice). Results are
// staged in shared memory and written out with coalesced stores (element-major, the layout the
// assembly gathers). Launch bounds hold it at 384 threads (6 blocks of 64) per SM: 168 registers,
// which the FP64 singular-G decision of the rare SVD path would otherwise raise to ~188.
template <int kT, bool kLinear>
__global__ void __launch_bounds__(kT, 384 / kT) k_element_f32(DevBody b, const double* __restrict__ xn,
															   const double* __restrict__ vn,
															   const double* __restrict__ xt,
															   const double* __restrict__ vt, float c2, float alpha,
															   float inv_dt, float* __restrict__ kslots,
															   float* __restrict__ rhsE, int* counters)
{
	// c2 = dt + beta, alpha and 1/dt arrive in FP32 from the host: formed in each thread they would
	// cost an FP64 add and an FP64 division per element.
	constexpr int kV = kSlots * 9;
	__shared__ float sks[kV][kT + 1];
	__shared__ float srhs[12][kT + 1];
	const int e0 = blockIdx.x * kT;
	const int e = e0 + threadIdx.x;
	const int E = b.E;
	if (e < E)
	{
		elem::ElemInF in;
		elem::gather_f32<kLinear>(b, e, xn, vn, xt, vt, c2, alpha, inv_dt, in);
		float g[4][3];
#pragma unroll
		for (int a = 0; a < 4; ++a)
#pragma unroll
			for (int k = 0; k < 3; ++k) g[a][k] = b.rest32[(3 * a + k) * E + e];
		const float lamV = b.rest32[13 * E + e], muV = b.rest32[14 * E + e], cm = b.rest32[15 * E + e];
		const int fl = elem::compute<float, false, elem::ElemInF, kLinear>(
			in, g, lamV, muV, cm, kslots ? &sks[0][threadIdx.x] : nullptr, kT + 1, &srhs[0][threadIdx.x], kT + 1,
			nullptr, nullptr);
		if (fl & 1) atomicAdd(&counters[1], 1);
		if (fl & 2) atomicAdd(&counters[0], 1);
	}
	__syncthreads();
	const int cnt = min(kT, E - e0);
	if (kslots)
	{
		// Split layout (k_assemble_f32): the first 8 values of element e's block k as one 32-byte
		// sector at kslots[8 (10 e + k)], the 9th at kslots[80 E + 10 e + k].
		float* dst8 = kslots + (size_t)e0 * (8 * kSlots);
		for (int idx = threadIdx.x; idx < cnt * 8 * kSlots; idx += kT)
		{
			const int el = idx / (8 * kSlots);
			const int j = idx - el * (8 * kSlots);
			dst8[idx] = sks[9 * (j >> 3) + (j & 7)][el];
		}
		float* dst1 = kslots + (size_t)E * (8 * kSlots) + (size_t)e0 * kSlots;
		for (int idx = threadIdx.x; idx < cnt * kSlots; idx += kT)
		{
			const int el = idx / kSlots;
			dst1[idx] = sks[9 * (idx - el * kSlots) + 8][el];
		}
	}
	float* dstR = rhsE + (size_t)e0 * 12;
	for (int idx = threadIdx.x; idx < cnt * 12; idx += kT)
	{
		const int el = idx / 12;
		dstR[idx] = srhs[idx - el * 12][el];
	}
}

// ------------------------------------------------------------------------------------------
// Assembly: one thread per lower block (I >= J). Sums element blocks in element order, forms
// S = c1 M + c2 K (c1 = 1/dt + alpha, c2 = dt + beta), applies boundary conditions
// (OdeState.cpp:197-218: zero rows and columns, diagonal 1) and writes the symmetric matrix
// that Eigen's selfadjointView<Lower> implies into its SELL-32 slots.
// ------------------------------------------------------------------------------------------
template <typename T>
__global__ void k_assemble(DevBody b, const T* __restrict__ ks, double c1, double c2, T* __restrict__ A,
						   T* __restrict__ invdiag)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	T s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	const int k1 = b.cptr[L + 1];
	for (int k = b.cptr[L]; k < k1; ++k)
	{
		const T* src = ks + (size_t)b.cidx[k] * 9;
#pragma unroll
		for (int m = 0; m < 9; ++m) s[m] += src[m];
	}
	const T mm = T(c1 * b.lmass[L]);
	const T c2t = T(c2);
	T blk[9];
#pragma unroll
	for (int m = 0; m < 9; ++m) blk[m] = c2t * s[m];
	blk[0] += mm;
	blk[4] += mm;
	blk[8] += mm;
	const int I = lb.x, J = lb.y;
	if (I == J)
	{
		blk[1] = blk[3];
		blk[2] = blk[6];
		blk[5] = blk[7];
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const int r = 3 * I + i, c = 3 * J + j;
			if (b.bc[r] | b.bc[c]) blk[3 * i + j] = (r == c) ? T(1) : T(0);
		}
#pragma unroll
	for (int m = 0; m < 9; ++m) A[(size_t)lb.z + 32 * m] = blk[m];
	if (lb.w >= 0)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) A[(size_t)lb.w + 32 * (3 * j + i)] = blk[3 * i + j];
	}
	if (I == J)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			const T d = blk[4 * i];
			invdiag[3 * I + i] = (d != T(0)) ? T(1) / d : T(1);  // DiagonalPreconditioner
		}
	}
}

// FP32 assembly from the FP32 element kernel's split layout: each contribution's first 8 values are
// one aligned 32-byte sector (two float4 loads), the 9th sits in the trailing array. The 36-byte blocks
// of the plain layout straddle sectors, so a contribution cost two sectors of reads there. Same sums,
// same order as k_assemble.
__global__ void k_assemble_f32(DevBody b, const float* __restrict__ ks, double c1, double c2, float* __restrict__ A,
							   float* __restrict__ invdiag)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	float s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	const float* ks1 = ks + (size_t)b.E * (8 * kSlots);
	const int k1 = b.cptr[L + 1];
	for (int k = b.cptr[L]; k < k1; ++k)
	{
		const int ci = b.cidx[k];
		const float4* src = reinterpret_cast<const float4*>(ks + (size_t)ci * 8);
		const float4 u = src[0], w = src[1];
		const float t = ks1[ci];
		s[0] += u.x;
		s[1] += u.y;
		s[2] += u.z;
		s[3] += u.w;
		s[4] += w.x;
		s[5] += w.y;
		s[6] += w.z;
		s[7] += w.w;
		s[8] += t;
	}
	const float mm = float(c1 * b.lmass[L]);
	const float c2t = float(c2);
	float blk[9];
#pragma unroll
	for (int m = 0; m < 9; ++m) blk[m] = c2t * s[m];
	blk[0] += mm;
	blk[4] += mm;
	blk[8] += mm;
	const int I = lb.x, J = lb.y;
	if (I == J)
	{
		blk[1] = blk[3];
		blk[2] = blk[6];
		blk[5] = blk[7];
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const int r = 3 * I + i, c = 3 * J + j;
			if (b.bc[r] | b.bc[c]) blk[3 * i + j] = (r == c) ? 1.f : 0.f;
		}
#pragma unroll
	for (int m = 0; m < 9; ++m) A[(size_t)lb.z + 32 * m] = blk[m];
	if (lb.w >= 0)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) A[(size_t)lb.w + 32 * (3 * j + i)] = blk[3 * i + j];
	}
	if (I == J)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			const float d = blk[4 * i];
			invdiag[3 * I + i] = (d != 0.f) ? 1.f / d : 1.f;  // DiagonalPreconditioner
		}
	}
}

template <typename T>
__global__ void k_rhs_gather(DevBody b, const T* __restrict__ rhsE, double g0, double g1, double g2, int gravityOn,
							 double* __restrict__ rhs, int applyBc)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= b.N) return;
	double s0 = 0, s1 = 0, s2 = 0;
	const int k1 = b.iptr[I + 1];
	if constexpr (std::is_same<T, float>::value)
	{
		// FP32 contributions summed exactly enough as float pairs (TwoSum; the errors' own sum keeps
		// ~2^-48 of the total) and converted to FP64 once: an FP64 add and conversion per contribution
		// (~140 FP64 instructions a node) would issue at 1/64 of the FP32 rate.
		float h[3] = {0.f, 0.f, 0.f}, l[3] = {0.f, 0.f, 0.f};
		for (int k = b.iptr[I]; k < k1; ++k)
		{
			const int c = b.iidx[k];
			const float* src = rhsE + (size_t)(c >> 2) * 12 + 3 * (c & 3);
#pragma unroll
			for (int i = 0; i < 3; ++i)
			{
				float t, e;
				elem::df_two_sum(h[i], src[i], t, e);
				h[i] = t;
				l[i] = __fadd_rn(l[i], e);
			}
		}
		s0 = double(h[0]) + double(l[0]);
		s1 = double(h[1]) + double(l[1]);
		s2 = double(h[2]) + double(l[2]);
	}
	else
	{
		for (int k = b.iptr[I]; k < k1; ++k)
		{
			const int c = b.iidx[k];
			const T* src = rhsE + (size_t)(c >> 2) * 12 + 3 * (c & 3);
			s0 += double(src[0]);
			s1 += double(src[1]);
			s2 += double(src[2]);
		}
	}
	if (gravityOn)  // FemRepresentation::addGravityForce (:641-662)
	{
		const double m = b.nmass[I];
		s0 += g0 * m;
		s1 += g1 * m;
		s2 += g2 * m;
	}
	if (applyBc)
	{
		if (b.bc[3 * I]) s0 = 0.0;
		if (b.bc[3 * I + 1]) s1 = 0.0;
		if (b.bc[3 * I + 2]) s2 = 0.0;
	}
	rhs[3 * I] = s0;
	rhs[3 * I + 1] = s1;
	rhs[3 * I + 2] = s2;
}

__global__ void k_assemble_full_csc(int nnz, const int* __restrict__ sptr, const int* __restrict__ sidx,
									const int* __restrict__ srow, const int* __restrict__ scol,
									const double* __restrict__ kfull, const double* __restrict__ smass,
									const uint8_t* __restrict__ bc, double c1, double c2, double* __restrict__ S)
{
	const int k = blockIdx.x * blockDim.x + threadIdx.x;
	if (k >= nnz) return;
	double s = 0;
	for (int t = sptr[k]; t < sptr[k + 1]; ++t) s += kfull[sidx[t]];
	double v = c1 * smass[k] + c2 * s;
	const int r = srow[k], c = scol[k];
	if (bc[r] | bc[c]) v = (r == c) ? 1.0 : 0.0;
	S[k] = v;
}

// ------------------------------------------------------------------------------------------
// Deterministic grid reductions: every block writes its partials, the last block to finish
// (ticket counter) sums them in block order. Results do not depend on scheduling. Per-thread and
// block-level sums use the accumulation type T; the cross-block sum is FP64.
// ------------------------------------------------------------------------------------------
struct OpSum
{
	template <typename T>
	__device__ static T apply(T a, T b) { return a + b; }
};
struct OpMax
{
	template <typename T>
	__device__ static T apply(T a, T b) { return a > b ? a : b; }
};

template <typename Op, typename T>
__device__ __forceinline__ T warp_reduce(T v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = Op::apply(v, __shfl_xor_sync(0xffffffffu, v, o));
	return v;
}

template <typename Op, int NV, typename T>
__device__ __forceinline__ void block_reduce(T (&v)[NV])
{
	__shared__ T sh[NV][32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
	for (int k = 0; k < NV; ++k) v[k] = warp_reduce<Op>(v[k]);
	__syncthreads();
	if (lane == 0)
#pragma unroll
		for (int k = 0; k < NV; ++k) sh[k][warp] = v[k];
	__syncthreads();
#pragma unroll
	for (int k = 0; k < NV; ++k)
	{
		const T x = (lane < nw) ? sh[k][lane] : T(0);
		v[k] = warp_reduce<Op>(x);  // every warp holds the block total
	}
}

// Returns true in every thread of the last block, with tot[] = grid totals (FP64).
template <typename Op, int NV, typename T>
__device__ bool grid_reduce(T (&v)[NV], double* part, unsigned int* ticket, double (&tot)[NV])
{
	__shared__ bool amLast;
	block_reduce<Op, NV, T>(v);
	if (threadIdx.x == 0)
	{
#pragma unroll
		for (int k = 0; k < NV; ++k) part[k * gridDim.x + blockIdx.x] = double(v[k]);
		__threadfence();
		const unsigned int t = atomicAdd(ticket, 1u);
		amLast = (t == gridDim.x - 1);
	}
	__syncthreads();
	if (!amLast) return false;
	__threadfence();
#pragma unroll
	for (int k = 0; k < NV; ++k)
	{
		double s = 0.0;
		for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s = Op::apply(s, __ldcg(&part[k * gridDim.x + i]));
		tot[k] = s;
	}
	block_reduce<Op, NV, double>(tot);
	if (threadIdx.x == 0) *ticket = 0u;
	return true;
}

// ------------------------------------------------------------------------------------------
// Sliced-ELL block SpMV: one thread per block row (3 scalar rows), no reductions, every value and
// column load coalesced across the warp (a warp is one chunk of 32 rows).
// ------------------------------------------------------------------------------------------
template <typename T, typename Acc, typename PT>
__device__ __forceinline__ void sell_row(const MatSellT<T>& A, const PT* __restrict__ p, int rs, Acc& a0, Acc& a1,
										 Acc& a2)
{
	const int c = rs >> 5, lane = rs & 31;
	const int k0 = A.off[c], k1 = A.off[c + 1];
	a0 = a1 = a2 = Acc(0);
	for (int k = k0; k < k1; ++k)
	{
		const int J = A.col[k * 32 + lane];
		const T* vb = A.val + (size_t)k * 288 + lane;
		const Acc p0 = Acc(p[3 * J]), p1 = Acc(p[3 * J + 1]), p2 = Acc(p[3 * J + 2]);
		a0 += Acc(vb[0]) * p0 + Acc(vb[32]) * p1 + Acc(vb[64]) * p2;
		a1 += Acc(vb[96]) * p0 + Acc(vb[128]) * p1 + Acc(vb[160]) * p2;
		a2 += Acc(vb[192]) * p0 + Acc(vb[224]) * p1 + Acc(vb[256]) * p2;
	}
}

// ------------------------------------------------------------------------------------------
// FP64 conjugate gradient (Eigen's conjugate_gradient with a Jacobi preconditioner, x0 = 0).
// ------------------------------------------------------------------------------------------
__global__ void k_cg_init(int n, const double* __restrict__ bvec, const double* __restrict__ invdiag,
						  double* __restrict__ x, double* __restrict__ r, double* __restrict__ p, CgCtl* ctl,
						  double* part, double tol, int maxIter)
{
	double v[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double bi = bvec[i];
		const double zi = invdiag[i] * bi;
		x[i] = 0.0;
		r[i] = bi;
		p[i] = zi;
		v[0] += bi * bi;
		v[1] += bi * zi;
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(v, part, &ctl->ticket[0], tot) && threadIdx.x == 0)
	{
		const double bb = tot[0];
		ctl->bb = bb;
		ctl->rz = tot[1];
		ctl->rr = bb;
		ctl->iter = 0;
		ctl->maxIter = maxIter;
		ctl->threshold = fmax(tol * tol * bb, DBL_MIN);
		ctl->converged = 1;
		ctl->done = (bb == 0.0 || bb < ctl->threshold) ? 1 : 0;
		if (!isfinite(bb))
		{
			ctl->done = 1;
			ctl->converged = 0;
		}
	}
}

__global__ void __launch_bounds__(256) k_cg_spmv_sell(MatSell3 A, const double* __restrict__ p,
													   double* __restrict__ q, CgCtl* ctl, double* part)
{
	if (ctl->done) return;
	double v[1] = {0.0};
	const int stride = gridDim.x * blockDim.x;
	const int nrowsPadded = (A.rows + 31) & ~31;
	for (int rs = blockIdx.x * blockDim.x + threadIdx.x; rs < nrowsPadded; rs += stride)
	{
		double a0, a1, a2;
		sell_row<double, double, double>(A, p, rs, a0, a1, a2);
		const int I = A.perm[rs];
		if (I >= 0)
		{
			q[3 * I] = a0;
			q[3 * I + 1] = a1;
			q[3 * I + 2] = a2;
			v[0] += p[3 * I] * a0 + p[3 * I + 1] * a1 + p[3 * I + 2] * a2;
		}
	}
	double tot[1];
	if (grid_reduce<OpSum, 1>(v, part, &ctl->ticket[1], tot) && threadIdx.x == 0)
	{
		ctl->pq = tot[0];
		ctl->alpha = ctl->rz / tot[0];
	}
}

__global__ void __launch_bounds__(256) k_cg_spmv_csr(MatCsr A, const double* __restrict__ p, double* __restrict__ q,
													  CgCtl* ctl, double* part)
{
	if (ctl->done) return;
	const int lane = threadIdx.x & 31;
	const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const int nwarps = (gridDim.x * blockDim.x) >> 5;
	double v[1] = {0.0};
	for (int row = warp; row < A.rows; row += nwarps)
	{
		double a = 0;
		for (int k = A.rowptr[row] + lane; k < A.rowptr[row + 1]; k += 32)
		{
			const int c = A.col[k];
			if ((unsigned)c < (unsigned)A.rows) a += A.val[k] * p[c];  // out-of-range columns are skipped
		}
		a = warp_reduce<OpSum>(a);
		if (lane == 0)
		{
			q[row] = a;
			v[0] += p[row] * a;
		}
	}
	double tot[1];
	if (grid_reduce<OpSum, 1>(v, part, &ctl->ticket[1], tot) && threadIdx.x == 0)
	{
		ctl->pq = tot[0];
		ctl->alpha = ctl->rz / tot[0];
	}
}

__global__ void k_cg_update(int n, const double* __restrict__ invdiag, const double* __restrict__ p,
							const double* __restrict__ q, double* __restrict__ x, double* __restrict__ r, CgCtl* ctl,
							double* part)
{
	if (ctl->done) return;
	const double alpha = ctl->alpha;
	double v[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		x[i] += alpha * p[i];
		const double ri = r[i] - alpha * q[i];
		r[i] = ri;
		v[0] += ri * ri;
		v[1] += ri * (invdiag[i] * ri);
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(v, part, &ctl->ticket[2], tot) && threadIdx.x == 0)
	{
		const double rr = tot[0];
		ctl->rr = rr;
		if (rr < ctl->threshold)
		{
			ctl->done = 1;
			ctl->converged = 1;
		}
		else if (!isfinite(rr))
		{
			ctl->done = 1;  // a NaN residual never converges; stop instead of running to maxIter
			ctl->converged = 0;
		}
		else
		{
			const double rzOld = ctl->rz;
			ctl->rz = tot[1];
			ctl->beta = tot[1] / rzOld;
			ctl->iter += 1;
			if (ctl->iter >= ctl->maxIter)
			{
				ctl->done = 1;
				ctl->converged = 0;
			}
		}
	}
}

__global__ void k_cg_pupdate(int n, const double* __restrict__ invdiag, const double* __restrict__ r,
							 double* __restrict__ p, const CgCtl* ctl)
{
	if (ctl->done) return;
	const double beta = ctl->beta;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		p[i] = invdiag[i] * r[i] + beta * p[i];
}

// ------------------------------------------------------------------------------------------
// State
// ------------------------------------------------------------------------------------------
// v_n += dv; x_n = x_t + dt v_n (OdeSolverEulerImplicit.cpp:98-99); optional Newton variation.
__global__ void k_state_update(int n, const double* __restrict__ dv, double* __restrict__ dvPrev,
							   const double* __restrict__ xt, double* __restrict__ xn, double* __restrict__ vn,
							   double dt, int trackNewton, CgCtl* ctl, double* part)
{
	double v[1] = {0.0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double d = dv[i];
		const double vi = vn[i] + d;
		vn[i] = vi;
		xn[i] = xt[i] + dt * vi;
		if (trackNewton)
		{
			v[0] = fmax(v[0], fabs(d - dvPrev[i]));
			dvPrev[i] = d;
		}
	}
	if (!trackNewton) return;
	double tot[1];
	if (grid_reduce<OpMax, 1>(v, part, &ctl->ticket[3], tot) && threadIdx.x == 0) ctl->newtonVar = tot[0];
}

// OdeState::isValid: the sums of positions and of velocities are finite (OdeState.cpp:268-278).
__global__ void k_validity(int n, const double* __restrict__ x, const double* __restrict__ v, CgCtl* ctl, double* part)
{
	double s[2] = {0, 0};
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		s[0] += x[i];
		s[1] += v[i];
	}
	double tot[2];
	if (grid_reduce<OpSum, 2>(s, part, &ctl->ticket[3], tot) && threadIdx.x == 0)
	{
		ctl->sumX = tot[0];
		ctl->sumV = tot[1];
		ctl->nonfinite = !(isfinite(tot[0]) && isfinite(tot[1]));
	}
}

__global__ void k_scatter_values(int count, const int* __restrict__ idx, const double* __restrict__ vals,
								 double* __restrict__ dst)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < count) dst[idx[i]] = vals[i];
}

// ------------------------------------------------------------------------------------------
// Multi-right-hand-side CG: the compliance columns (DeformableRepresentation::applyCompliance,
// DeformableRepresentation.cpp:175-191) solved together on the stored system. Each column follows
// Eigen's conjugate_gradient (Jacobi preconditioner, x0 = 0, stop at |r|^2 < tol^2 |b|^2 or maxIter)
// with its own scalars; one SpMM reads the matrix once per iteration for all columns.
// ------------------------------------------------------------------------------------------
constexpr int C8 = kMcgCols;

template <typename TD>
__global__ void k_mcg_init(int n, int ncols, const double* __restrict__ B, const uint8_t* __restrict__ bc,
						   const TD* __restrict__ invd, double* __restrict__ X, double* __restrict__ R,
						   double* __restrict__ Z, double* __restrict__ P, McgCtl* ctl, double* part, double tol,
						   int maxIter)
{
	double v[2 * C8];
#pragma unroll
	for (int k = 0; k < 2 * C8; ++k) v[k] = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double id = double(invd[i]);
#pragma unroll
		for (int c = 0; c < C8; ++c)
		{
			const size_t o = (size_t)i * C8 + c;
			const double b = (bc[i] || c >= ncols) ? 0.0 : B[o];
			const double z = id * b;
			R[o] = b;
			X[o] = 0.0;
			Z[o] = z;
			P[o] = z;
			v[c] += b * b;
			v[C8 + c] += b * z;
		}
	}
	double tot[2 * C8];
	if (grid_reduce<OpSum, 2 * C8>(v, part, &ctl->ticket[0], tot) && threadIdx.x == 0)
	{
		int all = 1;
		for (int c = 0; c < C8; ++c)
		{
			ctl->bb[c] = tot[c];
			ctl->rz[c] = tot[C8 + c];
			ctl->rr[c] = tot[c];
			ctl->threshold[c] = fmax(tol * tol * tot[c], DBL_MIN);
			ctl->iter[c] = 0;
			ctl->converged[c] = 1;
			ctl->done[c] = (c >= ncols || tot[c] == 0.0 || tot[c] < ctl->threshold[c] || !isfinite(tot[c])) ? 1 : 0;
			if (!isfinite(tot[c])) ctl->converged[c] = 0;
			ctl->alpha[c] = ctl->beta[c] = 0.0;
			all &= ctl->done[c];
		}
		ctl->maxIter = maxIter;
		ctl->allDone = all;
	}
}

template <typename T>
__global__ void k_mcg_spmm(MatSellT<T> A, const double* __restrict__ P, double* __restrict__ Q, McgCtl* ctl,
						   double* part)
{
	double v[C8];
#pragma unroll
	for (int c = 0; c < C8; ++c) v[c] = 0.0;
	for (int rs = blockIdx.x * blockDim.x + threadIdx.x; rs < A.rows; rs += gridDim.x * blockDim.x)
	{
		const int I = A.perm[rs];
		if (I < 0) continue;
		const int ch = rs >> 5, lane = rs & 31;
		double acc[3][C8];
#pragma unroll
		for (int m = 0; m < 3; ++m)
#pragma unroll
			for (int c = 0; c < C8; ++c) acc[m][c] = 0.0;
		const int k0 = A.off[ch], k1 = A.off[ch + 1];
		for (int k = k0; k < k1; ++k)
		{
			const int J = A.col[k * 32 + lane];
			const T* vb = A.val + (size_t)k * 288 + lane;
			double a[9];
#pragma unroll
			for (int m = 0; m < 9; ++m) a[m] = double(vb[32 * m]);
			const double* pj = P + (size_t)J * 3 * C8;
#pragma unroll
			for (int c = 0; c < C8; ++c)
			{
				const double p0 = pj[c], p1 = pj[C8 + c], p2 = pj[2 * C8 + c];
				acc[0][c] += a[0] * p0 + a[1] * p1 + a[2] * p2;
				acc[1][c] += a[3] * p0 + a[4] * p1 + a[5] * p2;
				acc[2][c] += a[6] * p0 + a[7] * p1 + a[8] * p2;
			}
		}
#pragma unroll
		for (int m = 0; m < 3; ++m)
#pragma unroll
			for (int c = 0; c < C8; ++c)
			{
				const size_t o = (size_t)(3 * I + m) * C8 + c;
				Q[o] = acc[m][c];
				v[c] += P[o] * acc[m][c];
			}
	}
	double tot[C8];
	if (grid_reduce<OpSum, C8>(v, part, &ctl->ticket[1], tot) && threadIdx.x == 0)
		for (int c = 0; c < C8; ++c)
		{
			ctl->pq[c] = tot[c];
			ctl->alpha[c] = ctl->done[c] ? 0.0 : ctl->rz[c] / tot[c];
		}
}

template <typename TD>
__global__ void k_mcg_update(int n, const TD* __restrict__ invd, const double* __restrict__ P,
							 const double* __restrict__ Q, double* __restrict__ X, double* __restrict__ R,
							 double* __restrict__ Z, McgCtl* ctl, double* part)
{
	double al[C8];
#pragma unroll
	for (int c = 0; c < C8; ++c) al[c] = ctl->alpha[c];
	double v[2 * C8];
#pragma unroll
	for (int k = 0; k < 2 * C8; ++k) v[k] = 0.0;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		const double id = double(invd[i]);
#pragma unroll
		for (int c = 0; c < C8; ++c)
		{
			const size_t o = (size_t)i * C8 + c;
			X[o] += al[c] * P[o];
			const double r = R[o] - al[c] * Q[o];
			R[o] = r;
			const double z = id * r;
			Z[o] = z;
			v[c] += r * r;
			v[C8 + c] += r * z;
		}
	}
	double tot[2 * C8];
	if (grid_reduce<OpSum, 2 * C8>(v, part, &ctl->ticket[2], tot) && threadIdx.x == 0)
	{
		int all = 1;
		for (int c = 0; c < C8; ++c)
		{
			if (!ctl->done[c])
			{
				ctl->rr[c] = tot[c];
				ctl->iter[c] += 1;
				if (tot[c] < ctl->threshold[c])
					ctl->done[c] = 1;
				else if (!isfinite(tot[c]) || ctl->iter[c] >= ctl->maxIter)
				{
					ctl->done[c] = 1;
					ctl->converged[c] = 0;
				}
				else
				{
					ctl->beta[c] = tot[C8 + c] / ctl->rz[c];
					ctl->rz[c] = tot[C8 + c];
				}
			}
			all &= ctl->done[c];
		}
		ctl->allDone = all;
	}
}

__global__ void k_mcg_pupdate(int n, const double* __restrict__ Z, double* __restrict__ P, const McgCtl* ctl)
{
	double be[C8];
	int dn[C8];
#pragma unroll
	for (int c = 0; c < C8; ++c)
	{
		be[c] = ctl->beta[c];
		dn[c] = ctl->done[c];
	}
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
#pragma unroll
		for (int c = 0; c < C8; ++c)
		{
			const size_t o = (size_t)i * C8 + c;
			if (!dn[c]) P[o] = Z[o] + be[c] * P[o];
		}
}

// Rotation of every element at positions x (the polar factor of the corotational update).
__global__ void k_element_rotation(DevBody b, const double* __restrict__ x, double* __restrict__ Re)
{
	const int e = blockIdx.x * blockDim.x + threadIdx.x;
	if (e >= b.E) return;
	const int E = b.E;
	const int4 t4 = b.tets[e];
	const int nd[4] = {t4.x, t4.y, t4.z, t4.w};
	double F[9];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			double s = 0.0;
#pragma unroll
			for (int a = 1; a < 4; ++a) s += (x[3 * nd[a] + i] - x[3 * nd[0] + i]) * b.rest[(3 * a + j) * E + e];
			F[3 * i + j] = s;
		}
	double R[9];
	if (!elem::polar_newton(F, R)) elem::polar_svd(F, R);
#pragma unroll
	for (int k = 0; k < 9; ++k) Re[(size_t)e * 9 + k] = R[k];
}

// Unit quaternion (w, x, y, z) of a rotation matrix (row-major), by the largest of the four
// diagonal combinations (numerically stable for every rotation).
__device__ void quat_from_matrix(const double* R, double* q)
{
	const double t = R[0] + R[4] + R[8];
	if (t > 0.0)
	{
		const double s = 2.0 * sqrt(1.0 + t);
		q[0] = 0.25 * s;
		q[1] = (R[7] - R[5]) / s;
		q[2] = (R[2] - R[6]) / s;
		q[3] = (R[3] - R[1]) / s;
	}
	else if (R[0] > R[4] && R[0] > R[8])
	{
		const double s = 2.0 * sqrt(1.0 + R[0] - R[4] - R[8]);
		q[0] = (R[7] - R[5]) / s;
		q[1] = 0.25 * s;
		q[2] = (R[1] + R[3]) / s;
		q[3] = (R[2] + R[6]) / s;
	}
	else if (R[4] > R[8])
	{
		const double s = 2.0 * sqrt(1.0 + R[4] - R[0] - R[8]);
		q[0] = (R[2] - R[6]) / s;
		q[1] = (R[1] + R[3]) / s;
		q[2] = 0.25 * s;
		q[3] = (R[5] + R[7]) / s;
	}
	else
	{
		const double s = 2.0 * sqrt(1.0 + R[8] - R[0] - R[4]);
		q[0] = (R[3] - R[1]) / s;
		q[1] = (R[2] + R[6]) / s;
		q[2] = (R[5] + R[7]) / s;
		q[3] = 0.25 * s;
	}
}

__device__ void matrix_from_quat(const double* q, double* R)
{
	const double w = q[0], x = q[1], y = q[2], z = q[3];
	R[0] = 1 - 2 * (y * y + z * z);
	R[1] = 2 * (x * y - w * z);
	R[2] = 2 * (x * z + w * y);
	R[3] = 2 * (x * y + w * z);
	R[4] = 1 - 2 * (x * x + z * z);
	R[5] = 2 * (y * z - w * x);
	R[6] = 2 * (x * z - w * y);
	R[7] = 2 * (y * z + w * x);
	R[8] = 1 - 2 * (x * x + y * y);
}

// Spherical linear interpolation from a to b at t along the shorter arc (linear weights when the
// quaternions are within one rounding unit of each other).
__device__ void quat_slerp(const double* a, const double* b, double t, double* out)
{
	const double d = a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
	const double ad = fabs(d);
	double s0, s1;
	if (ad >= 1.0 - DBL_EPSILON)
	{
		s0 = 1.0 - t;
		s1 = t;
	}
	else
	{
		const double th = acos(ad), st = sin(th);
		s0 = sin((1.0 - t) * th) / st;
		s1 = sin(t * th) / st;
	}
	if (d < 0.0) s1 = -s1;
#pragma unroll
	for (int k = 0; k < 4; ++k) out[k] = s0 * a[k] + s1 * b[k];
}

__global__ void k_node_rotation(DevBody b, const double* __restrict__ Re, double* __restrict__ Wn)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= b.N) return;
	const int k0 = b.iptr[I], k1 = b.iptr[I + 1];
	double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
	if (k1 > k0)
	{
		double q[4];
		quat_from_matrix(Re + (size_t)(b.iidx[k0] >> 2) * 9, q);
		for (int k = k0 + 1; k < k1; ++k)
		{
			double qe[4], qn[4];
			quat_from_matrix(Re + (size_t)(b.iidx[k] >> 2) * 9, qe);
			const double i = double(k - k0 + 1);  // the element's 1-based position at this node
			quat_slerp(q, qe, 1.0 - 1.0 / i, qn);
#pragma unroll
			for (int m = 0; m < 4; ++m) q[m] = qn[m];
		}
		matrix_from_quat(q, R);
	}
#pragma unroll
	for (int m = 0; m < 9; ++m) Wn[(size_t)I * 9 + m] = R[m];
}

__global__ void k_apply_node_rotation(int N, const double* __restrict__ Wn, double* __restrict__ X, int transpose)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= N * C8) return;
	const int I = t / C8, c = t % C8;
	const double* W = Wn + (size_t)I * 9;
	const size_t o = (size_t)3 * I * C8 + c;
	const double x0 = X[o], x1 = X[o + C8], x2 = X[o + 2 * C8];
	for (int i = 0; i < 3; ++i)
	{
		const double r = transpose ? (W[i] * x0 + W[3 + i] * x1 + W[6 + i] * x2)
								   : (W[3 * i] * x0 + W[3 * i + 1] * x1 + W[3 * i + 2] * x2);
		X[o + i * C8] = r;
	}
}

__global__ void k_prev_positions(int n, const double* __restrict__ x, const double* __restrict__ v, double dt,
								 double* __restrict__ out)
{
	const int i = blockIdx.x * blockDim.x + threadIdx.x;
	if (i < n) out[i] = x[i] - dt * v[i];
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------------------------------------
// Launchers
// ------------------------------------------------------------------------------------------
void launch_element_fp64(const DevBody& b, const double* xn, const double* vn, const double* xt, const double* vt,
						 double dt, double alpha, double beta, double* kslots, double* rhsE, double* kfull,
						 double* fE, int* counters, cudaStream_t s, bool linear)
{
	if (b.E == 0) return;
	const int nb = blocks(b.E, kElemThreads);
	if (kfull)
	{
		if (linear)
			k_element_fp64<true, true><<<nb, kElemThreads, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE,
																	kfull, fE, counters);
		else
			k_element_fp64<true, false><<<nb, kElemThreads, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE,
																	 kfull, fE, counters);
	}
	else if (linear)
		k_element_fp64<false, true><<<nb, kElemThreads, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE,
																 nullptr, nullptr, counters);
	else
		k_element_fp64<false, false><<<nb, kElemThreads, 0, s>>>(b, xn, vn, xt, vt, dt, alpha, beta, kslots, rhsE,
																  nullptr, nullptr, counters);
}

int launch_element_f32(const DevBody& b, const double* xn, const double* vn, const double* xt, const double* vt,
					   double dt, double alpha, double beta, float* kslots, float* rhsE, int* counters,
					   cudaStream_t s, int elemsPerBlock, bool linear)
{
	if (b.E == 0) return 0;
	const float c2f = float(dt + beta), alphaf = float(alpha), invdtf = float(1.0 / dt);
	int kernels = 1;
	if (!linear)
	{
		k_node_prep<<<blocks(b.n, 256), 256, 0, s>>>(b.n, xn, vn, xt, vt, (xt == xn) && (vt == vn), b.nodeX, b.nodeV,
													 b.nodeDx, b.nodeDv);
		kernels = 2;
	}
	if (elemsPerBlock == 32)
	{
		if (linear)
			k_element_f32<32, true><<<blocks(b.E, 32), 32, 0, s>>>(b, xn, vn, xt, vt, c2f, alphaf, invdtf, kslots, rhsE,
																	counters);
		else
			k_element_f32<32, false><<<blocks(b.E, 32), 32, 0, s>>>(b, xn, vn, xt, vt, c2f, alphaf, invdtf, kslots, rhsE,
																	 counters);
	}
	else if (linear)
		k_element_f32<64, true><<<blocks(b.E, 64), 64, 0, s>>>(b, xn, vn, xt, vt, c2f, alphaf, invdtf, kslots, rhsE,
																counters);
	else
		k_element_f32<64, false><<<blocks(b.E, 64), 64, 0, s>>>(b, xn, vn, xt, vt, c2f, alphaf, invdtf, kslots, rhsE,
																 counters);
	return kernels;
}

void launch_assemble(const DevBody& b, const double* kslots, double c1, double c2, double* A, double* invdiag,
					 cudaStream_t s)
{
	if (b.nl == 0) return;
	k_assemble<double><<<blocks(b.nl, 128), 128, 0, s>>>(b, kslots, c1, c2, A, invdiag);
}

void launch_assemble(const DevBody& b, const float* kslots, double c1, double c2, float* A, float* invdiag,
					 cudaStream_t s)
{
	if (b.nl == 0) return;
	k_assemble_f32<<<blocks(b.nl, 128), 128, 0, s>>>(b, kslots, c1, c2, A, invdiag);
}

void launch_rhs_gather(const DevBody& b, const double* rhsE, const double* gravity, int gravityOn, double* rhs,
					   int applyBc, cudaStream_t s)
{
	if (b.N == 0) return;
	k_rhs_gather<double><<<blocks(b.N, 128), 128, 0, s>>>(b, rhsE, gravity[0], gravity[1], gravity[2], gravityOn, rhs,
														  applyBc);
}

void launch_rhs_gather(const DevBody& b, const float* rhsE, const double* gravity, int gravityOn, double* rhs,
					   int applyBc, cudaStream_t s)
{
	if (b.N == 0) return;
	k_rhs_gather<float><<<blocks(b.N, 128), 128, 0, s>>>(b, rhsE, gravity[0], gravity[1], gravity[2], gravityOn, rhs,
														 applyBc);
}

void launch_assemble_full_csc(int nnz, const int* sptr, const int* sidx, const int* srow, const int* scol,
							  const double* kfull, const double* smass, const uint8_t* bc, double c1, double c2,
							  double* S, cudaStream_t s)
{
	if (nnz == 0) return;
	k_assemble_full_csc<<<blocks(nnz, 256), 256, 0, s>>>(nnz, sptr, sidx, srow, scol, kfull, smass, bc, c1, c2, S);
}

void launch_cg_init(int n, const double* b, const double* invdiag, double* x, double* r, double* p, CgCtl* ctl,
					double* part, double tol, int maxIter, const Launch& L)
{
	k_cg_init<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, b, invdiag, x, r, p, ctl, part, tol, maxIter);
}

void launch_cg_spmv_sell(const MatSell3& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_spmv_sell<<<L.vecGrid, 256, 0, L.stream>>>(A, p, q, ctl, part);
}

void launch_cg_spmv_csr(const MatCsr& A, const double* p, double* q, CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_spmv_csr<<<L.vecGrid, 256, 0, L.stream>>>(A, p, q, ctl, part);
}

void launch_cg_update(int n, const double* invdiag, const double* p, const double* q, double* x, double* r,
					  CgCtl* ctl, double* part, const Launch& L)
{
	k_cg_update<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invdiag, p, q, x, r, ctl, part);
}

void launch_cg_pupdate(int n, const double* invdiag, const double* r, double* p, CgCtl* ctl, const Launch& L)
{
	k_cg_pupdate<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invdiag, r, p, ctl);
}

void launch_state_update(int n, const double* dv, double* dvPrev, const double* xt, double* xn, double* vn,
						 double dt, int trackNewton, CgCtl* ctl, double* part, const Launch& L)
{
	k_state_update<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, dv, dvPrev, xt, xn, vn, dt, trackNewton, ctl, part);
}

void launch_validity(int n, const double* x, const double* v, CgCtl* ctl, double* part, const Launch& L)
{
	k_validity<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, x, v, ctl, part);
}

void launch_scatter_values(int count, const int* idx, const double* vals, double* dst, cudaStream_t s)
{
	if (count <= 0) return;
	k_scatter_values<<<blocks(count, 256), 256, 0, s>>>(count, idx, vals, dst);
}

void launch_mcg_init(int n, int ncols, const double* B, const uint8_t* bc, const double* invd64, const float* invd32,
					 double* X, double* R, double* Z, double* P, McgCtl* ctl, double* part, double tol, int maxIter,
					 const Launch& L)
{
	if (invd64)
		k_mcg_init<double><<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, ncols, B, bc, invd64, X, R, Z, P, ctl, part, tol,
																	 maxIter);
	else
		k_mcg_init<float><<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, ncols, B, bc, invd32, X, R, Z, P, ctl, part, tol,
																	maxIter);
}

void launch_mcg_spmm(const MatSellT<double>* A64, const MatSellT<float>* A32, const double* P, double* Q,
					 McgCtl* ctl, double* part, const Launch& L)
{
	if (A64)
		k_mcg_spmm<double><<<L.vecGrid, kVecThreads, 0, L.stream>>>(*A64, P, Q, ctl, part);
	else
		k_mcg_spmm<float><<<L.vecGrid, kVecThreads, 0, L.stream>>>(*A32, P, Q, ctl, part);
}

void launch_mcg_update(int n, const double* invd64, const float* invd32, const double* P, const double* Q, double* X,
					   double* R, double* Z, McgCtl* ctl, double* part, const Launch& L)
{
	if (invd64)
		k_mcg_update<double><<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invd64, P, Q, X, R, Z, ctl, part);
	else
		k_mcg_update<float><<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, invd32, P, Q, X, R, Z, ctl, part);
}

void launch_mcg_pupdate(int n, const double* Z, double* P, const McgCtl* ctl, const Launch& L)
{
	k_mcg_pupdate<<<L.vecGrid, kVecThreads, 0, L.stream>>>(n, Z, P, ctl);
}

void launch_element_rotation(const DevBody& b, const double* x, double* Re, cudaStream_t s)
{
	if (b.E == 0) return;
	k_element_rotation<<<blocks(b.E, 128), 128, 0, s>>>(b, x, Re);
}

void launch_node_rotation(const DevBody& b, const double* Re, double* Wn, cudaStream_t s)
{
	if (b.N == 0) return;
	k_node_rotation<<<blocks(b.N, 128), 128, 0, s>>>(b, Re, Wn);
}

void launch_apply_node_rotation(int N, const double* Wn, double* X, bool transpose, cudaStream_t s)
{
	if (N == 0) return;
	k_apply_node_rotation<<<blocks((long long)N * C8, 256), 256, 0, s>>>(N, Wn, X, transpose ? 1 : 0);
}

void launch_prev_positions(int n, const double* x, const double* v, double dt, double* out, cudaStream_t s)
{
	if (n == 0) return;
	k_prev_positions<<<blocks(n, 256), 256, 0, s>>>(n, x, v, dt, out);
}


namespace {

// One thread per external block: adds D + dt K into the system the CG reads (lower block and its
// mirror; the diagonal block through its lower triangle), leaving boundary rows and columns as the
// boundary conditions set them, and refreshes the Jacobi diagonal of a diagonal block.
template <typename T>
__global__ void k_ext_system(int count, const ExtBlock* __restrict__ blocks, const uint8_t* __restrict__ bc,
							 T* __restrict__ A, T* __restrict__ invdiag)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= count) return;
	const ExtBlock& e = blocks[t];
#pragma unroll
	for (int i = 0; i < 3; ++i)
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const int r = 3 * e.I + i, c = 3 * e.J + j;
			if (bc[r] | bc[c]) continue;
			if (e.I == e.J)
				A[(size_t)e.z + 32 * (3 * i + j)] += T(i >= j ? e.v[3 * i + j] : e.v[3 * j + i]);
			else
			{
				A[(size_t)e.z + 32 * (3 * i + j)] += T(e.v[3 * i + j]);
				A[(size_t)e.w + 32 * (3 * j + i)] += T(e.v[3 * i + j]);
			}
		}
	if (e.I == e.J)
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			if (bc[3 * e.I + i]) continue;
			const T d = A[(size_t)e.z + 32 * (4 * i)];
			invdiag[3 * e.I + i] = (d != T(0)) ? T(1) / d : T(1);
		}
}

__global__ void k_ext_rhs(int count, const ExtRow* __restrict__ rows, const ExtCol* __restrict__ cols,
						  const uint8_t* __restrict__ bc, const double* __restrict__ xn, const double* __restrict__ xt,
						  const double* __restrict__ vn, double dt, double* __restrict__ rhs)
{
	const int t = blockIdx.x * blockDim.x + threadIdx.x;
	if (t >= count) return;
	const ExtRow& r = rows[t];
	double acc[3] = {r.F[0], r.F[1], r.F[2]};
	for (int k = r.k0; k < r.k1; ++k)
	{
		const ExtCol& c = cols[k];
		double u[3];
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const int d = 3 * c.J + j;
			u[j] = (xn[d] - xt[d]) - dt * vn[d];
		}
#pragma unroll
		for (int i = 0; i < 3; ++i) acc[i] += c.K[3 * i] * u[0] + c.K[3 * i + 1] * u[1] + c.K[3 * i + 2] * u[2];
	}
#pragma unroll
	for (int i = 0; i < 3; ++i)
		if (!bc[3 * r.I + i]) rhs[3 * r.I + i] += acc[i];
}

}  // namespace

void launch_ext_system(int count, const ExtBlock* ext, const uint8_t* bc, double* A, double* invdiag, cudaStream_t s)
{
	if (count > 0) k_ext_system<double><<<blocks(count, 128), 128, 0, s>>>(count, ext, bc, A, invdiag);
}

void launch_ext_system(int count, const ExtBlock* ext, const uint8_t* bc, float* A, float* invdiag, cudaStream_t s)
{
	if (count > 0) k_ext_system<float><<<blocks(count, 128), 128, 0, s>>>(count, ext, bc, A, invdiag);
}

void launch_ext_rhs(int count, const ExtRow* rows, const ExtCol* cols, const uint8_t* bc, const double* xn,
					const double* xt, const double* vn, double dt, double* rhs, cudaStream_t s)
{
	if (count > 0) k_ext_rhs<<<blocks(count, 128), 128, 0, s>>>(count, rows, cols, bc, xn, xt, vn, dt, rhs);
}

}  // namespace gbfem
