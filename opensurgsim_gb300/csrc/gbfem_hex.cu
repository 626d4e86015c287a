// gbfem_hex.cu -- sm_103a kernels of the hexahedral (Fem3DElementCube) implicit-Euler step.
//
// Fem3DElementCube is a linear element: its K and M (2x2x2 Gauss-Legendre quadrature at the rest
// state, Fem3DElementCube.cpp:97-167, 267-319) never change, and its force is f = -K (x - x0)
// (:129-141). So the step keeps the assembled K (3x3 blocks) and the scalar mass of every block
// resident in HBM in the SELL-32 layout of the system matrix and
//   * forms S = (1/dt + alpha) M + (dt + beta) K with the boundary conditions once per dt
//     (k_system_from_k), and
//   * forms each step's right-hand side in one pass over K and M (k_hex_rhs, after k_hex_uw has
//     formed the two per-node vectors it needs), reading them through L2:
//       rhs = f(x_n, v_n) + K (x_n - x_t - dt v_n) - M (v_n - v_t) / dt
//           = -K (x_t - x0 + (dt + beta) v_n) - M (alpha v_n + (v_n - v_t) / dt) + g m_lumped
//     (OdeSolverEulerImplicit.cpp:124-161 with FemRepresentation::computeFMDK, :479-545; x_n cancels).
// The element integrals run once, one CTA slice of 64 threads per element: 64 threads evaluate
// the shape-function gradients at the 8 Gauss points of their element into shared memory, then 36
// of them form one lower-triangle node block each (8 diagonal blocks and 28 node pairs).

#include <cstdint>

#include "gbfem_internal.h"

namespace gbfem {

namespace {

constexpr int kHexThreads = 64;     // threads per element in k_hex_element
constexpr int kHexPerCta = 4;       // elements per CTA

inline int blocks_for(int n, int t) { return (n + t - 1) / t; }

// Shape-function signs of the 8 corners (Fem3DElementCube.cpp:72-74).
__device__ __forceinline__ double hex_sign(int axis, int a)
{
	// eps: - + + - - + + -   eta: - - + + - - + +   mu: - - - - + + + +
	const int bit = axis == 0 ? (((a + 1) >> 1) & 1) : (axis == 1 ? ((a >> 1) & 1) : ((a >> 2) & 1));
	return bit ? 1.0 : -1.0;
}

// Slot s of an 8-node element: s < 8 is the diagonal block of node s, then the 28 pairs a < b in
// lexicographic order.
__device__ __forceinline__ void hex_slot_pair(int s, int& a, int& b)
{
	if (s < 8)
	{
		a = b = s;
		return;
	}
	int p = s - 8;
	a = 0;
	while (p >= 7 - a)
	{
		p -= 7 - a;
		++a;
	}
	b = a + 1 + p;
}

__global__ void __launch_bounds__(kHexThreads * kHexPerCta)
	k_hex_element(int E, const int* __restrict__ nodes, const double* __restrict__ xrest,
				  const double* __restrict__ young, const double* __restrict__ poisson, const double* __restrict__ rho,
				  double* __restrict__ slots, double* __restrict__ smass)
{
	__shared__ double sg[kHexPerCta][8][8][3];  // [element][Gauss point][node] spatial gradient
	__shared__ double sN[kHexPerCta][8][8];     // shape-function values
	__shared__ double sw[kHexPerCta][8];        // det J (weights are 1)
	const int le = threadIdx.x / kHexThreads, t = threadIdx.x % kHexThreads;
	const int e = blockIdx.x * kHexPerCta + le;
	const bool live = e < E;
	if (live)
	{
		// Thread t: Gauss point gp = t / 8, node a = t % 8. Points +1/sqrt(3) then -1/sqrt(3) per
		// axis, loops eps (slowest), eta, mu (GaussLegendreQuadrature.cpp:30-34, Fem3DElementCube.cpp:113-126).
		const int gp = t >> 3, a = t & 7;
		const double q = 0.57735026918962576451;  // 1/sqrt(3)
		const double xi[3] = {(gp & 4) ? -q : q, (gp & 2) ? -q : q, (gp & 1) ? -q : q};
		double J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
		for (int i = 0; i < 8; ++i)
		{
			const int nd = nodes[8 * (size_t)e + i];
			const double s0 = hex_sign(0, i), s1 = hex_sign(1, i), s2 = hex_sign(2, i);
			const double o0 = 1 + xi[0] * s0, o1 = 1 + xi[1] * s1, o2 = 1 + xi[2] * s2;
			const double d[3] = {0.125 * s0 * o1 * o2, 0.125 * o0 * s1 * o2, 0.125 * o0 * o1 * s2};
			const double p[3] = {xrest[3 * (size_t)nd], xrest[3 * (size_t)nd + 1], xrest[3 * (size_t)nd + 2]};
#pragma unroll
			for (int r = 0; r < 3; ++r)
#pragma unroll
				for (int c = 0; c < 3; ++c) J[r][c] += p[c] * d[r];
		}
		const double c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
		const double c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
		const double c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
		const double det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
		const double id = 1.0 / det;  // the host has checked |det| > 1e-12 at every Gauss point
		const double Ji[3][3] = {{c00 * id, (J[0][2] * J[2][1] - J[0][1] * J[2][2]) * id, (J[0][1] * J[1][2] - J[0][2] * J[1][1]) * id},
								 {c01 * id, (J[0][0] * J[2][2] - J[0][2] * J[2][0]) * id, (J[0][2] * J[1][0] - J[0][0] * J[1][2]) * id},
								 {c02 * id, (J[0][1] * J[2][0] - J[0][0] * J[2][1]) * id, (J[0][0] * J[1][1] - J[0][1] * J[1][0]) * id}};
		const double s0 = hex_sign(0, a), s1 = hex_sign(1, a), s2 = hex_sign(2, a);
		const double o0 = 1 + xi[0] * s0, o1 = 1 + xi[1] * s1, o2 = 1 + xi[2] * s2;
		const double d[3] = {0.125 * s0 * o1 * o2, 0.125 * o0 * s1 * o2, 0.125 * o0 * o1 * s2};
#pragma unroll
		for (int r = 0; r < 3; ++r) sg[le][gp][a][r] = Ji[r][0] * d[0] + Ji[r][1] * d[1] + Ji[r][2] * d[2];
		sN[le][gp][a] = 0.125 * o0 * o1 * o2;
		if (a == 0) sw[le][gp] = det;
	}
	__syncthreads();
	if (!live || t >= 36) return;
	int a, b;
	hex_slot_pair(t, a, b);
	const int na = nodes[8 * (size_t)e + a], nb = nodes[8 * (size_t)e + b];
	const double nu = poisson[e], Ey = young[e];
	const double lambda = Ey * nu / ((1.0 + nu) * (1.0 - 2.0 * nu));
	const double mu = Ey / (2.0 * (1 + nu));
	// The block is stored with the larger global node id as its row: K_ab or its transpose K_ba.
	const int r = (na >= nb) ? a : b, c = (na >= nb) ? b : a;
	double k[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	double m = 0.0;
	for (int gp = 0; gp < 8; ++gp)
	{
		const double w = sw[le][gp];
		const double gr[3] = {sg[le][gp][r][0], sg[le][gp][r][1], sg[le][gp][r][2]};
		const double gc[3] = {sg[le][gp][c][0], sg[le][gp][c][1], sg[le][gp][c][2]};
		const double dot = gr[0] * gc[0] + gr[1] * gc[1] + gr[2] * gc[2];
		// (B_r^T C B_c)(i,j) = lambda g_r,i g_c,j + mu g_r,j g_c,i + mu delta_ij (g_r . g_c)
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
				k[3 * i + j] += w * (lambda * gr[i] * gc[j] + mu * gr[j] * gc[i] + (i == j ? mu * dot : 0.0));
		m += w * rho[e] * sN[le][gp][r] * sN[le][gp][c];
	}
	double* dst = slots + ((size_t)e * 36 + t) * 9;
#pragma unroll
	for (int i = 0; i < 9; ++i) dst[i] = k[i];
	smass[(size_t)e * 36 + t] = m;
}

// One thread per lower block: K and the scalar mass of the block summed over its element slots in
// element order, written to both SELL positions of the block (the mirror transposed).
__global__ void k_assemble_k(DevBody b, const double* __restrict__ slots, const double* __restrict__ smass,
							 double* __restrict__ K, double* __restrict__ Ms, double* __restrict__ lmass)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	double s[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
	double m = 0.0;
	for (int k = b.cptr[L]; k < b.cptr[L + 1]; ++k)
	{
		const int c = b.cidx[k];
		const double* src = slots + (size_t)c * 9;
#pragma unroll
		for (int i = 0; i < 9; ++i) s[i] += src[i];
		m += smass[c];
	}
	lmass[L] = m;
#pragma unroll
	for (int i = 0; i < 9; ++i) K[(size_t)lb.z + 32 * i] = s[i];
	Ms[(size_t)(lb.z / 288) * 32 + lb.z % 288] = m;
	if (lb.w >= 0)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) K[(size_t)lb.w + 32 * (3 * j + i)] = s[3 * i + j];
		Ms[(size_t)(lb.w / 288) * 32 + lb.w % 288] = m;
	}
}

// Mass lumping (FemRepresentation::computeFMDK, FemRepresentation.cpp:499-508: every row of M summed
// onto its diagonal, the rest of the row zeroed, the pattern kept). Pass 1, one thread per SELL row:
// the row's scalar block masses summed (padding slots hold zero) into rowsum[I], every slot of the
// row zeroed. Pass 2, one thread per lower block: the diagonal block gets the row sum back, and the
// lower-block masses S is formed from become the row sums on the diagonal and zero elsewhere.
__global__ void k_hex_lump_rows(MatSell3 K, double* __restrict__ Ms, double* __restrict__ rowsum)
{
	const int rs = blockIdx.x * blockDim.x + threadIdx.x;
	if (rs >= K.rows) return;
	const int I = K.perm[rs];
	if (I < 0) return;
	const int c = rs >> 5, lane = rs & 31;
	double m = 0.0;
	for (int k = K.off[c]; k < K.off[c + 1]; ++k) m += Ms[k * 32 + lane];
	for (int k = K.off[c]; k < K.off[c + 1]; ++k) Ms[k * 32 + lane] = 0.0;
	rowsum[I] = m;
}

__global__ void k_hex_lump_lower(DevBody b, const double* __restrict__ rowsum, double* __restrict__ Ms,
								 double* __restrict__ lmass)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	if (lb.x != lb.y)
	{
		lmass[L] = 0.0;
		return;
	}
	const double m = rowsum[lb.x];
	lmass[L] = m;
	Ms[(size_t)(lb.z / 288) * 32 + lb.z % 288] = m;
}

// S = c1 M + c2 K from the stored K (its lower block) with the boundary conditions, as k_assemble.
template <typename T>
__global__ void k_system_from_k(DevBody b, const double* __restrict__ K, double c1, double c2, T* __restrict__ A,
								T* __restrict__ invdiag)
{
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= b.nl) return;
	const int4 lb = b.lblk[L];
	const double mm = c1 * b.lmass[L];
	double blk[9];
#pragma unroll
	for (int i = 0; i < 9; ++i) blk[i] = c2 * K[(size_t)lb.z + 32 * i];
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
			if (b.bc[r] | b.bc[c]) blk[3 * i + j] = (r == c) ? 1.0 : 0.0;
		}
#pragma unroll
	for (int i = 0; i < 9; ++i) A[(size_t)lb.z + 32 * i] = T(blk[i]);
	if (lb.w >= 0)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j) A[(size_t)lb.w + 32 * (3 * j + i)] = T(blk[3 * i + j]);
	}
	if (I == J)
	{
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			const T d = T(blk[4 * i]);
			invdiag[3 * I + i] = (d != T(0)) ? T(1) / d : T(1);  // DiagonalPreconditioner
		}
	}
}

// Per node: u = (x_t - x0) + (dt + beta) v_n and w = alpha v_n + (v_n - v_t) / dt, one 48-byte
// record (u, w) per node, so the matrix pass below gathers one record per block column and spends
// only its 12 FMAs per block on FP64 arithmetic (FP64 issues at 1/64 of the FP32 rate here).
__global__ void k_hex_uw(int N, const double* __restrict__ xrest, const double* __restrict__ xt,
						 const double* __restrict__ vn, const double* __restrict__ vt, double alpha, double c2,
						 double inv_dt, double2* __restrict__ uw)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= N) return;
	double u[3], w[3];
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		const double v = vn[3 * I + i];
		u[i] = (xt[3 * I + i] - xrest[3 * I + i]) + c2 * v;
		w[i] = alpha * v + (v - vt[3 * I + i]) * inv_dt;
	}
	uw[3 * (size_t)I] = make_double2(u[0], u[1]);
	uw[3 * (size_t)I + 1] = make_double2(u[2], w[0]);
	uw[3 * (size_t)I + 2] = make_double2(w[1], w[2]);
}

// rhs = -(K u + M w) + g m_lumped with the boundary rows zeroed. One thread per SELL row (a warp is
// one chunk of 32 rows: every K value, mass and column load is coalesced).
__global__ void __launch_bounds__(256)
	k_hex_rhs(MatSell3 K, const double* __restrict__ Ms, const double2* __restrict__ uw,
			  const double* __restrict__ nmass, const uint8_t* __restrict__ bc, double g0, double g1, double g2,
			  int gravityOn, double* __restrict__ rhs)
{
	const int rs = blockIdx.x * blockDim.x + threadIdx.x;
	if (rs >= K.rows) return;
	const int I = K.perm[rs];
	if (I < 0) return;
	const int c = rs >> 5, lane = rs & 31;
	double a0 = 0.0, a1 = 0.0, a2 = 0.0;
	for (int k = K.off[c]; k < K.off[c + 1]; ++k)
	{
		const int J = K.col[k * 32 + lane];
		const double* kb = K.val + (size_t)k * 288 + lane;
		const double m = Ms[k * 32 + lane];
		const double2 r0 = uw[3 * (size_t)J], r1 = uw[3 * (size_t)J + 1], r2 = uw[3 * (size_t)J + 2];
		a0 += kb[0] * r0.x + kb[32] * r0.y + kb[64] * r1.x + m * r1.y;
		a1 += kb[96] * r0.x + kb[128] * r0.y + kb[160] * r1.x + m * r2.x;
		a2 += kb[192] * r0.x + kb[224] * r0.y + kb[256] * r1.x + m * r2.y;
	}
	double r0 = -a0, r1 = -a1, r2 = -a2;
	if (gravityOn)  // FemRepresentation::addGravityForce (:641-662), lumped rho V / 8 per node
	{
		const double mI = nmass[I];
		r0 += g0 * mI;
		r1 += g1 * mI;
		r2 += g2 * mI;
	}
	rhs[3 * I] = bc[3 * I] ? 0.0 : r0;
	rhs[3 * I + 1] = bc[3 * I + 1] ? 0.0 : r1;
	rhs[3 * I + 2] = bc[3 * I + 2] ? 0.0 : r2;
}

// ---- Mixed form: the same right-hand side without FP64 in the matrix pass (FP64 issues at 1/64 of
// the FP32 rate here, and the FP64 pass is bound by it). K and the slot masses are stored once as
// unevaluated float pairs hi + lo (~2^-48 relative), u and w per node likewise; the pass forms each
// product's rounding error by FMA, adds the terms of a row by TwoSum and renormalises the pair once
// a block, so the row sums keep ~2^-44 of the terms' magnitude (the rows' cancellation against
// gravity, added in FP64 at the end, stays exact enough for the mixed solve's refinement).

__device__ __forceinline__ void hex_two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// (sh, sl) += a * b for float pairs a, b (the lo * lo term is below the pair's precision).
__device__ __forceinline__ void hex_acc(float& sh, float& sl, float2 a, float2 b)
{
	const float P = __fmul_rn(a.x, b.x);
	const float e = __fmaf_rn(a.x, b.x, -P);
	const float cross = __fmaf_rn(a.x, b.y, __fmul_rn(a.y, b.x));
	float t, et;
	hex_two_sum(sh, P, t, et);
	sh = t;
	sl = __fadd_rn(sl, __fadd_rn(et, __fadd_rn(e, cross)));
}

__global__ void k_split_pairs(size_t n, const double* __restrict__ src, float2* __restrict__ dst)
{
	const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const double v = src[i];
	const float hi = float(v);
	dst[i] = make_float2(hi, float(v - double(hi)));
}

// u = x_t - x0 + (dt + beta) v_n and w = alpha v_n + (v_n - v_t) / dt in FP64, stored as float pairs:
// three float4 per node {u0, u1}, {u2, w0}, {w1, w2}.
__global__ void k_hex_uw_df(int N, const double* __restrict__ xrest, const double* __restrict__ xt,
							const double* __restrict__ vn, const double* __restrict__ vt, double alpha, double c2,
							double inv_dt, float4* __restrict__ uw)
{
	const int I = blockIdx.x * blockDim.x + threadIdx.x;
	if (I >= N) return;
	float h[6], l[6];
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		const double v = vn[3 * I + i];
		const double u = (xt[3 * I + i] - xrest[3 * I + i]) + c2 * v;
		const double w = alpha * v + (v - vt[3 * I + i]) * inv_dt;
		h[i] = float(u);
		l[i] = float(u - double(h[i]));
		h[3 + i] = float(w);
		l[3 + i] = float(w - double(h[3 + i]));
	}
	uw[3 * (size_t)I] = make_float4(h[0], l[0], h[1], l[1]);
	uw[3 * (size_t)I + 1] = make_float4(h[2], l[2], h[3], l[3]);
	uw[3 * (size_t)I + 2] = make_float4(h[4], l[4], h[5], l[5]);
}

__global__ void __launch_bounds__(256)
	k_hex_rhs_df(MatSell3 K, const float2* __restrict__ Kp, const float2* __restrict__ Msp,
				 const float4* __restrict__ uw, const double* __restrict__ nmass, const uint8_t* __restrict__ bc,
				 double g0, double g1, double g2, int gravityOn, double* __restrict__ rhs)
{
	const int rs = blockIdx.x * blockDim.x + threadIdx.x;
	if (rs >= K.rows) return;
	const int I = K.perm[rs];
	if (I < 0) return;
	const int c = rs >> 5, lane = rs & 31;
	float sh[3] = {0.f, 0.f, 0.f}, sl[3] = {0.f, 0.f, 0.f};
	for (int k = K.off[c]; k < K.off[c + 1]; ++k)
	{
		const int J = K.col[k * 32 + lane];
		const float2* kb = Kp + (size_t)k * 288 + lane;
		const float2 m = Msp[k * 32 + lane];
		const float4 r0 = uw[3 * (size_t)J], r1 = uw[3 * (size_t)J + 1], r2 = uw[3 * (size_t)J + 2];
		const float2 u[3] = {make_float2(r0.x, r0.y), make_float2(r0.z, r0.w), make_float2(r1.x, r1.y)};
		const float2 w[3] = {make_float2(r1.z, r1.w), make_float2(r2.x, r2.y), make_float2(r2.z, r2.w)};
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
#pragma unroll
			for (int j = 0; j < 3; ++j) hex_acc(sh[i], sl[i], kb[32 * (3 * i + j)], u[j]);
			hex_acc(sh[i], sl[i], m, w[i]);
			float t, e;
			hex_two_sum(sh[i], sl[i], t, e);
			sh[i] = t;
			sl[i] = e;
		}
	}
	double r[3];
#pragma unroll
	for (int i = 0; i < 3; ++i) r[i] = -(double(sh[i]) + double(sl[i]));
	if (gravityOn)  // FemRepresentation::addGravityForce (:641-662), lumped rho V / 8 per node
	{
		const double mI = nmass[I];
		r[0] += g0 * mI;
		r[1] += g1 * mI;
		r[2] += g2 * mI;
	}
#pragma unroll
	for (int i = 0; i < 3; ++i) rhs[3 * I + i] = bc[3 * I + i] ? 0.0 : r[i];
}

}  // namespace

void launch_split_pairs(size_t n, const double* src, float2* dst, cudaStream_t s)
{
	if (n == 0) return;
	k_split_pairs<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, src, dst);
}

void launch_hex_rhs_df(const MatSell3& K, const float2* Kp, const float2* Msp, const DevBody& b, const double* xt,
					   const double* vn, const double* vt, double dt, double alpha, double beta, const double* gravity,
					   int gravityOn, double* uw, double* rhs, cudaStream_t s)
{
	if (K.rows == 0) return;
	float4* uw4 = reinterpret_cast<float4*>(uw);  // 48 bytes per node, 16-byte aligned allocation
	k_hex_uw_df<<<blocks_for(b.N, 256), 256, 0, s>>>(b.N, b.xrest, xt, vn, vt, alpha, dt + beta, 1.0 / dt, uw4);
	k_hex_rhs_df<<<blocks_for(K.rows, 256), 256, 0, s>>>(K, Kp, Msp, uw4, b.nmass, b.bc, gravity[0], gravity[1],
														 gravity[2], gravityOn, rhs);
}

void launch_hex_element(int E, const int* nodes, const double* xrest, const double* young, const double* poisson,
						const double* rho, double* slots, double* smass, cudaStream_t s)
{
	if (E == 0) return;
	k_hex_element<<<blocks_for(E, kHexPerCta), kHexThreads * kHexPerCta, 0, s>>>(E, nodes, xrest, young, poisson,
																				  rho, slots, smass);
}

void launch_assemble_k(const DevBody& b, const double* slots, const double* smass, double* K, double* Ms,
					   double* lmass, cudaStream_t s)
{
	if (b.nl == 0) return;
	k_assemble_k<<<blocks_for(b.nl, 128), 128, 0, s>>>(b, slots, smass, K, Ms, lmass);
}

void launch_hex_lump_masses(const DevBody& b, const MatSell3& K, double* Ms, double* lmass, double* rowsum,
							cudaStream_t s)
{
	if (b.nl == 0 || K.rows == 0) return;
	k_hex_lump_rows<<<blocks_for(K.rows, 256), 256, 0, s>>>(K, Ms, rowsum);
	k_hex_lump_lower<<<blocks_for(b.nl, 128), 128, 0, s>>>(b, rowsum, Ms, lmass);
}

void launch_system_from_k(const DevBody& b, const double* K, double c1, double c2, double* A, double* invdiag,
						  cudaStream_t s)
{
	if (b.nl == 0) return;
	k_system_from_k<double><<<blocks_for(b.nl, 128), 128, 0, s>>>(b, K, c1, c2, A, invdiag);
}

void launch_system_from_k(const DevBody& b, const double* K, double c1, double c2, float* A, float* invdiag,
						  cudaStream_t s)
{
	if (b.nl == 0) return;
	k_system_from_k<float><<<blocks_for(b.nl, 128), 128, 0, s>>>(b, K, c1, c2, A, invdiag);
}

void launch_hex_rhs(const MatSell3& K, const double* Ms, const DevBody& b, const double* xt, const double* vn,
					const double* vt, double dt, double alpha, double beta, const double* gravity, int gravityOn,
					double* uw, double* rhs, cudaStream_t s)
{
	if (K.rows == 0) return;
	double2* uw2 = reinterpret_cast<double2*>(uw);  // 6 doubles per node, 16-byte aligned allocation
	k_hex_uw<<<blocks_for(b.N, 256), 256, 0, s>>>(b.N, b.xrest, xt, vn, vt, alpha, dt + beta, 1.0 / dt, uw2);
	k_hex_rhs<<<blocks_for(K.rows, 256), 256, 0, s>>>(K, Ms, uw2, b.nmass, b.bc, gravity[0], gravity[1], gravity[2],
													  gravityOn, rhs);
}

}  // namespace gbfem
