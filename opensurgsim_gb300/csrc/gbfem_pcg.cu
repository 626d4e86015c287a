// gbfem_pcg.cu -- persistent mixed-precision CG over a batch of independent systems (segments).
//
// One cooperative launch runs a whole solve for every segment (mesh) of a batch: FP32 CG
// iterations on the FP32 SELL-32 matrix with per-segment scalars, the solution accumulated as a
// float pair hi + lo (~48 bits; FP32 deltas folded at each refresh), and per-segment "reliable
// updates": when a segment's FP32 residual has dropped by `drop` since its last refresh (or looks
// converged), its true residual b - A x is recomputed in double-float arithmetic (FP64 products
// would run at 1/64 of the FP32 rate) and convergence is decided on it, at the same
// |r|^2 < tol^2 |b|^2 rule as the FP64 form (Eigen's ConjugateGradient).
//
// Work is cut into chunks of 32 matrix rows (one node row per lane); segments own contiguous
// chunk ranges. In the two-phase CG schedule every iteration has two phases separated by grid
// barriers: phase 1 is the SpMV (or, for a segment due for a refresh, the true residual), phase 2
// the row-local update (or the rescale after a refresh). The one-phase schedule (Chronopoulos and
// Gear's recurrences) does an iteration's SpMV, row update and both dot products in one phase. Each
// phase walks only the chunks of the segments still iterating (the active set), split over the CTAs
// by exact integer arithmetic on cumulative weights: SpMV phases balance block columns, row-local
// phases chunk counts. Every CTA recomputes its own range whenever the active set changes, so no CTA
// idles on finished meshes. The plain FP64 form (Eigen's CG on the FP64 values) runs the two-phase
// structure without refreshes.
//
// Per-segment sums are deterministic: each CTA sums its chunk partials of a segment in chunk
// order; a segment spread over CTAs bf..bl is completed by the last of them to arrive (ticket
// counter), which adds the CTAs' partials in a fixed order. A grid-barrier wait gives up after a
// wall-time limit (1 s in the solve): the kernel records an error and returns (the host reports
// GBFEM_CUDA_ERROR).

#include <cfloat>
#include <cstdint>

#include "gbfem_pcg.h"

namespace gbfem {
namespace {

constexpr unsigned kFull = 0xffffffffu;
// Backstop on the polls of one barrier wait (each poll is an L2 round trip plus a short sleep);
// the wall-time limit (PcgArgs::barrierTimeoutNs) ends a wait first.
constexpr long long kSpinLimit = 50000000LL;
constexpr int kWarps = kPcgThreads / 32;

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p)
{
	unsigned v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
	return v;
}

__device__ __forceinline__ unsigned atom_add_acq_rel(unsigned* p, unsigned v)
{
	unsigned old;
	asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
	return old;
}

__device__ __forceinline__ void red_add_release(unsigned* p, unsigned v)
{
	asm volatile("red.release.gpu.global.add.u32 [%0], %1;" : : "l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ int ldi(const int* p) { return *(const volatile int*)p; }
__device__ __forceinline__ double ldd(const double* p) { return *(const volatile double*)p; }
__device__ __forceinline__ double2 ldv2(const double* p)  // 16-byte aligned
{
	double2 v;
	asm volatile("ld.volatile.global.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "l"(p));
	return v;
}
// {beta, mode} of a segment in one load.
__device__ __forceinline__ void load_beta_mode(const SegCtl* S, double& beta, int& mode)
{
	const double2 v = ldv2(&S->beta);
	beta = v.x;
	mode = (int)(unsigned)(__double_as_longlong(v.y) & 0xffffffffLL);
}

__device__ __forceinline__ unsigned long long global_ns()
{
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}

// Grid-wide barrier ending phase `ph` (all blocks co-resident: cooperative launch). The last
// block to arrive clears the event counters that phase ph + 1 will count into.
// A waiting block gives up after `timeoutNs` of wall time (or kSpinLimit polls, whichever comes
// first), records the error in g->err and returns false. Once g->err is set every block returns
// false from its next barrier, and a block already waiting stops within 1024 polls.
__device__ bool grid_barrier(PcgGlobal* g, int ph, long long timeoutNs)
{
	__syncthreads();
	__shared__ int ok;
	if (threadIdx.x == 0)
	{
		ok = 1;
		const unsigned gen = ld_acquire(&g->barGen);
		// Arrival releases this block's writes (ordered before by __syncthreads) and, for the last
		// block, acquires everyone else's before it releases the next generation.
		if (atom_add_acq_rel(&g->barCount, 1u) == gridDim.x - 1)
		{
			g->finishedIn[(ph + 1) & 1] = 0;
			g->refreshIn[(ph + 1) & 1] = 0;
			g->barCount = 0;
			red_add_release(&g->barGen, 1u);
		}
		else
		{
			const unsigned long long t0 = global_ns();
			long long spins = 0;
			while (ld_acquire(&g->barGen) == gen)
			{
				if (++spins > kSpinLimit || (long long)(global_ns() - t0) > timeoutNs ||
					((spins & 1023) == 0 && ldi(&g->err)))
				{
					atomicExch(&g->err, 1);
					ok = 0;
					break;
				}
				__nanosleep(32);
			}
		}
		// Acquire side (the spin's ld.acquire): the other blocks' writes of the finished phase are
		// visible to this block, whose next phase reads the vectors with plain, L1-cached loads.
	}
	__syncthreads();
	return ok && !*(volatile int*)&g->err;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
	return v;
}

// Largest s in [0, nseg) with Cp[s] <= t (for t < Cp[nseg] that segment is non-empty).
__device__ __forceinline__ int seg_of(const int* Cp, int nseg, int t)
{
	int lo = 0, hi = nseg - 1;
	while (lo < hi)
	{
		const int mid = (lo + hi + 1) >> 1;
		if (Cp[mid] <= t)
			lo = mid;
		else
			hi = mid - 1;
	}
	return lo;
}

// Warp-collective lower bound: smallest i in [L, R) with arr[i] >= key, or R. Same result in
// every lane. Each round probes 32 evenly spaced entries.
__device__ int lower_bound_warp(const int* __restrict__ arr, int L, int R, int key)
{
	const int lane = threadIdx.x & 31;
	while (R - L > 32)
	{
		const int step = (R - L + 31) / 32;
		const int i = L + (lane + 1) * step - 1;
		const bool pred = (i < R) ? (__ldg(&arr[i]) >= key) : true;
		const unsigned m = __ballot_sync(kFull, pred);
		const int k = __ffs(m) - 1;  // m != 0: the last probe is at or past R - 1
		const int iPrev = L + k * step - 1;
		const int iK = L + (k + 1) * step - 1;
		L = (k == 0) ? L : iPrev + 1;
		R = (iK < R) ? iK : R;
	}
	const int i = L + lane;
	const bool pred = (i < R) && (__ldg(&arr[i]) >= key);
	const unsigned m = __ballot_sync(kFull, pred);
	return m ? L + __ffs(m) - 1 : R;
}

// Per-CTA view of a set of segments: chunk-count prefix Cp and weight prefix Wp over the
// segments (inactive segments count zero), and the partition range of this CTA.
struct SetView
{
	const int* Cp;
	const int* Wp;   // null for chunk-count partitions
	int lo, hi;      // this CTA's positions
	int n;           // total positions
	long long tot;   // total weight (== n for chunk-count partitions)
};

// First position of CTA b in a block-column-weighted partition: the smallest t with
// Wc(t) * G >= tot * b, where Wc(t) is the weight of positions [0, t). Warp-collective.
__device__ int weighted_start(const PcgArgs& a, const int* Cp, const int* Wp, const int* sc, int nseg, int b, int G)
{
	const long long tot = Wp[nseg];
	if (b <= 0 || tot == 0) return 0;
	if (b >= G) return Cp[nseg];
	const long long X = tot * b;
	int lo = 0, hi = nseg - 1;  // largest s with Wp[s] * G < X
	while (lo < hi)
	{
		const int mid = (lo + hi + 1) >> 1;
		if ((long long)Wp[mid] * G < X)
			lo = mid;
		else
			hi = mid - 1;
	}
	const int s = lo;
	const int c0 = sc[s], ns = sc[s + 1] - sc[s];
	const long long base = __ldg(&a.cumW[c0]);
	const long long mult = (Wp[s + 1] - Wp[s]) / (__ldg(&a.cumW[c0 + ns]) - base);  // segment weight multiplier
	const long long need = (X - (long long)Wp[s] * G + G * mult - 1) / (G * mult);  // >= 1
	const int key = (int)(base + need);
	int j = lower_bound_warp(a.cumW, c0 + 1, c0 + ns + 1, key) - c0;
	j = min(j, ns);
	return Cp[s] + j;
}

// The CTA holding a position of cumulative weight w: floor(w * G / tot), capped.
__device__ __forceinline__ int cta_of(long long w, long long tot, int G)
{
	return (int)min((long long)(G - 1), (w * G) / tot);
}

// First and last CTA holding positions of non-empty segment s in view V.
__device__ __forceinline__ int2 seg_ctas(const PcgArgs& a, const SetView& V, const int* sc, int s)
{
	const int G = gridDim.x;
	if (!V.Wp) return make_int2(cta_of(V.Cp[s], V.n, G), cta_of(V.Cp[s + 1] - 1, V.n, G));
	const int c0 = sc[s], cl = sc[s + 1] - 1;
	const long long mult = (V.Wp[s + 1] - V.Wp[s]) / (__ldg(&a.cumW[cl + 1]) - __ldg(&a.cumW[c0]));
	const long long wl = (long long)V.Wp[s + 1] - mult * (__ldg(&a.cumW[cl + 1]) - __ldg(&a.cumW[cl]));
	return make_int2(cta_of(V.Wp[s], V.tot, G), cta_of(wl, V.tot, G));
}

// Calls f(slot, s, c) for the CTA's positions [lo, hi): slot = t - lo, s the segment and c the
// chunk of position t. Warps take the next position from a shared counter (zeroed before the
// phase), so a warp that drew short chunks takes more of them; the results do not depend on
// which warp ran a position (partials are kept per slot and summed in slot order).
template <typename F>
__device__ __forceinline__ void for_chunks(const SetView& V, const int* sc, int nseg, int* next, F f)
{
	const int lane = threadIdx.x & 31;
	for (;;)
	{
		int k = 0;
		if (lane == 0) k = atomicAdd(next, 1);
		const int t = V.lo + __shfl_sync(kFull, k, 0);
		if (t >= V.hi) return;
		const int s = seg_of(V.Cp, nseg, t);
		f(t - V.lo, s, sc[s] + (t - V.Cp[s]));
	}
}

// Reduce this CTA's chunk partials per segment (sp[k * M + slot]) and complete segments across
// CTAs; fin(s, totals) runs once per segment, in lane 0 of one warp (or thread 0) of the completing
// CTA. The segments of the CTA's range are independent: warp w takes the range's segments w, w + 8, ...
// A segment spread over CTAs bf..bl is completed by the last of them to arrive (ticket), which adds
// the CTAs' partials in a fixed order: in the arriving warp when they are few (at most two a lane),
// else by all threads of the CTA in one round of loads (one large mesh spans every CTA of the grid:
// one warp would need several dependent rounds of L2 loads on the path to the grid barrier).
template <int NV, typename Fin>
__device__ void reduce_segments(const PcgArgs& a, const SetView& V, const int* sc, const double* sp, Fin fin)
{
	__syncthreads();
	const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
	const int nseg = a.nsegs, G = gridDim.x, B = blockIdx.x, M = a.maxChunksPerCta;
	// Wide segments this CTA completes (at most two: the first and the last of its range).
	__shared__ int shWideN;
	__shared__ int shWideS[2];
	__shared__ int2 shWideFl[2];
	__shared__ double shWarpSum[kPcgNV][kWarps];
	if (threadIdx.x == 0) shWideN = 0;
	__syncthreads();
	auto arrive = [&](int s, int2 fl, const double* v) {
		const int which = (B > fl.x) ? 0 : 1;  // 0: first slot (CTAs after bf), 1: last slot (bf)
		unsigned tk = 0;
		if (lane == 0)
		{
#pragma unroll
			for (int k = 0; k < NV; ++k) a.slots[(size_t)(2 * k + which) * G + B] = v[k];
			tk = atom_add_acq_rel(&a.seg[s].ticket, 1u);  // releases the slot, acquires the others'
		}
		tk = __shfl_sync(kFull, tk, 0);
		if (tk != (unsigned)(fl.y - fl.x)) return;
		if (fl.y - fl.x > 64)
		{
			if (lane == 0)
			{
				const int i = atomicAdd(&shWideN, 1);
				if (i < 2)
				{
					shWideS[i] = s;
					shWideFl[i] = fl;
				}
				else
					atomicExch(&a.g->err, 2);  // cannot happen (a range has one first and one last segment)
			}
			return;
		}
		__syncwarp();
		// The CTAs' partials, lane l adding CTAs bf + 1 + l, bf + 33 + l in that order, all loads issued
		// before they are added.
		double u[NV], t[NV], tot[NV];
		const int b0 = fl.x + 1 + lane, b1 = b0 + 32;
#pragma unroll
		for (int k = 0; k < NV; ++k)
		{
			u[k] = (lane == 0) ? __ldcg(&a.slots[(size_t)(2 * k + 1) * G + fl.x]) : 0.0;
			t[k] = (b0 <= fl.y) ? __ldcg(&a.slots[(size_t)(2 * k) * G + b0]) : 0.0;
			tot[k] = (b1 <= fl.y) ? __ldcg(&a.slots[(size_t)(2 * k) * G + b1]) : 0.0;
		}
#pragma unroll
		for (int k = 0; k < NV; ++k) tot[k] = warp_sum((u[k] + t[k]) + tot[k]);
		if (lane == 0)
		{
			a.seg[s].ticket = 0u;
			fin(s, tot);
		}
	};
	if (V.lo < V.hi)
	{
		for (int s = seg_of(V.Cp, nseg, V.lo) + wid; s < nseg && V.Cp[s] < V.hi; s += kWarps)
		{
			if (V.Cp[s + 1] == V.Cp[s]) continue;
			const int t0 = max(V.lo, V.Cp[s]), t1 = min(V.hi, V.Cp[s + 1]);
			double v[NV];
#pragma unroll
			for (int k = 0; k < NV; ++k)
			{
				double u = 0.0;
				for (int t = t0 + lane; t < t1; t += 32) u += sp[k * M + (t - V.lo)];
				v[k] = warp_sum(u);
			}
			const int2 fl = seg_ctas(a, V, sc, s);
			if (fl.x == fl.y)
			{
				if (lane == 0) fin(s, v);
			}
			else
				arrive(s, fl, v);
		}
	}
	else if (V.lo < V.n && wid == 0)
	{
		// An empty range strictly inside a segment still counts among that segment's CTAs.
		const int s = seg_of(V.Cp, nseg, V.lo);
		if (V.lo > V.Cp[s])
		{
			double v[NV];
#pragma unroll
			for (int k = 0; k < NV; ++k) v[k] = 0.0;
			arrive(s, seg_ctas(a, V, sc, s), v);
		}
	}
	__syncthreads();
	const int nWide = min(shWideN, 2);
	if (nWide == 0) return;
	// The ticket's acquire was made by one thread; every thread of the CTA reads the other CTAs' slots.
	__threadfence();
	for (int i = 0; i < nWide; ++i)
	{
		const int s = shWideS[i];
		const int2 fl = shWideFl[i];
		// Thread j adds CTAs bf + 1 + j, bf + 1 + j + 256, ...; thread 0 starts from bf's slot; the warps'
		// sums are added in warp order: a fixed order whatever the timing.
		double u[NV];
#pragma unroll
		for (int k = 0; k < NV; ++k) u[k] = (threadIdx.x == 0) ? __ldcg(&a.slots[(size_t)(2 * k + 1) * G + fl.x]) : 0.0;
		for (int b = fl.x + 1 + threadIdx.x; b <= fl.y; b += kPcgThreads)
#pragma unroll
			for (int k = 0; k < NV; ++k) u[k] += __ldcg(&a.slots[(size_t)(2 * k) * G + b]);
#pragma unroll
		for (int k = 0; k < NV; ++k)
		{
			const double w = warp_sum(u[k]);
			if (lane == 0) shWarpSum[k][wid] = w;
		}
		__syncthreads();
		if (threadIdx.x == 0)
		{
			double tot[NV];
#pragma unroll
			for (int k = 0; k < NV; ++k)
			{
				tot[k] = 0.0;
#pragma unroll
				for (int w = 0; w < kWarps; ++w) tot[k] += shWarpSum[k][w];
			}
			a.seg[s].ticket = 0u;
			fin(s, tot);
		}
		__syncthreads();
	}
}

// q[row] (3 floats) = sum over the chunk's SELL slots of A_block * p(J), with p(J) = z(J) + beta p_old(J)
// formed on the fly from the packed records; four slots' loads are issued before any is used. The
// matrix (values, columns) is read once per pass with the streaming hint (evict first), so L2 keeps
// the gathered z/p records, which rows a mesh layer apart reuse.
__device__ __forceinline__ void spmv_row_zp(const PcgArgs& a, const float4* __restrict__ zp, int c, int lane,
											float beta, float& a0, float& a1, float& a2)
{
	const int k0 = __ldg(&a.off[c]), k1 = __ldg(&a.off[c + 1]);
	int k = k0;
	// Column indices are loaded one round ahead of the gathers they address, so a round waits on the
	// gathers alone, not on a column load and then the gathers.
	int Jn[4] = {0, 0, 0, 0};
#pragma unroll
	for (int u = 0; u < 4; ++u)
		if (k + u < k1) Jn[u] = __ldcs(&a.col[(k + u) * 32 + lane]);
	for (; k + 4 <= k1; k += 4)
	{
		int J[4];
#pragma unroll
		for (int u = 0; u < 4; ++u) J[u] = Jn[u];
#pragma unroll
		for (int u = 0; u < 4; ++u)
			if (k + 4 + u < k1) Jn[u] = __ldcs(&a.col[(k + 4 + u) * 32 + lane]);
		float4 zj[4], pj[4];
#pragma unroll
		for (int u = 0; u < 4; ++u)
		{
			zj[u] = zp[2 * J[u]];
			pj[u] = zp[2 * J[u] + 1];
		}
#pragma unroll
		for (int u = 0; u < 4; ++u)
		{
			const float* vb = a.val + (size_t)(k + u) * 288 + lane;
			const float p0 = zj[u].x + beta * pj[u].x, p1 = zj[u].y + beta * pj[u].y, p2 = zj[u].z + beta * pj[u].z;
			a0 += __ldcs(vb) * p0 + __ldcs(vb + 32) * p1 + __ldcs(vb + 64) * p2;
			a1 += __ldcs(vb + 96) * p0 + __ldcs(vb + 128) * p1 + __ldcs(vb + 160) * p2;
			a2 += __ldcs(vb + 192) * p0 + __ldcs(vb + 224) * p1 + __ldcs(vb + 256) * p2;
		}
	}
	// The last 1 to 3 slots (their columns already in Jn) in one round as well (the count is the same
	// in every lane), instead of one dependent column -> record -> value chain each.
	const int rem = k1 - k;
	if (rem > 0)
	{
		float4 zj[3], pj[3];
#pragma unroll
		for (int u = 0; u < 3; ++u)
			if (u < rem)
			{
				zj[u] = zp[2 * Jn[u]];
				pj[u] = zp[2 * Jn[u] + 1];
			}
#pragma unroll
		for (int u = 0; u < 3; ++u)
			if (u < rem)
			{
				const float* vb = a.val + (size_t)(k + u) * 288 + lane;
				const float p0 = zj[u].x + beta * pj[u].x, p1 = zj[u].y + beta * pj[u].y, p2 = zj[u].z + beta * pj[u].z;
				a0 += __ldcs(vb) * p0 + __ldcs(vb + 32) * p1 + __ldcs(vb + 64) * p2;
				a1 += __ldcs(vb + 96) * p0 + __ldcs(vb + 128) * p1 + __ldcs(vb + 160) * p2;
				a2 += __ldcs(vb + 192) * p0 + __ldcs(vb + 224) * p1 + __ldcs(vb + 256) * p2;
			}
	}
}

// FP64 form: the same product on the FP64 values, p(J) = z(J) + beta p_old(J) from the 64-byte
// records {z0 z1 | z2 - | p0 p1 | p2 -}; two slots' loads issued before either is used (four need
// 124 registers, or spill at three CTAs per SM).
__device__ __forceinline__ void spmv_row_zp64(const PcgArgs& a, const double2* __restrict__ zp, int c, int lane,
											  double beta, double& a0, double& a1, double& a2)
{
	const int k0 = __ldg(&a.off[c]), k1 = __ldg(&a.off[c + 1]);
	for (int k = k0; k < k1; k += 2)
	{
		const int nk = min(2, k1 - k);
		int J[2];
#pragma unroll
		for (int u = 0; u < 2; ++u)
			if (u < nk) J[u] = __ldcs(&a.col[(k + u) * 32 + lane]);
		double2 r0[2], r1[2], r2[2], r3[2];
#pragma unroll
		for (int u = 0; u < 2; ++u)
			if (u < nk)
			{
				r0[u] = zp[4 * J[u]];
				r1[u] = zp[4 * J[u] + 1];
				r2[u] = zp[4 * J[u] + 2];
				r3[u] = zp[4 * J[u] + 3];
			}
#pragma unroll
		for (int u = 0; u < 2; ++u)
			if (u < nk)
			{
				const double* vb = a.val64 + (size_t)(k + u) * 288 + lane;
				const double p0 = r0[u].x + beta * r2[u].x, p1 = r0[u].y + beta * r2[u].y, p2 = r1[u].x + beta * r3[u].x;
				a0 += __ldcs(vb) * p0 + __ldcs(vb + 32) * p1 + __ldcs(vb + 64) * p2;
				a1 += __ldcs(vb + 96) * p0 + __ldcs(vb + 128) * p1 + __ldcs(vb + 160) * p2;
				a2 += __ldcs(vb + 192) * p0 + __ldcs(vb + 224) * p1 + __ldcs(vb + 256) * p2;
			}
	}
}

// kPcgMixed1: a row's next residual and preconditioned residual from its record {r, d0}, {w, d1},
// {s, d2} (d = invdiag): s' = w + beta s (= A p), r' = r - alpha s', u' = d r'. The owning row and
// every row that gathers it call this one function, with explicit roundings, so all of them form
// bit-identical u' and the SpMV multiplies exactly the vector whose dot products the owner takes.
__device__ __forceinline__ void cg1_next(const float4& R, const float4& W, const float4& S, float al, float be,
										 float& s0, float& s1, float& s2, float& r0, float& r1, float& r2, float& u0,
										 float& u1, float& u2)
{
	s0 = __fmaf_rn(be, S.x, W.x);
	s1 = __fmaf_rn(be, S.y, W.y);
	s2 = __fmaf_rn(be, S.z, W.z);
	r0 = __fmaf_rn(-al, s0, R.x);
	r1 = __fmaf_rn(-al, s1, R.y);
	r2 = __fmaf_rn(-al, s2, R.z);
	u0 = __fmul_rn(R.w, r0);
	u1 = __fmul_rn(W.w, r1);
	u2 = __fmul_rn(S.w, r2);
}

// kPcgMixed1, CG step: w[row] (3 floats) = sum over the chunk's SELL slots of A_block * u'(J), u'(J)
// formed by cg1_next from the neighbour's 48-byte record. Rounds of U slots: the columns of the next
// round are loaded while this round's records are gathered, and the round's matrix values are loaded
// together with its records, so a round waits on one memory latency (values loaded after the records
// are gathered made each round two: one large mesh's solve 19.8 -> 17.2 ms; where the phases stream
// nearly the whole batch this order is slower, 41.5 -> 53.1 ms, and the autotuner runs that batch
// in the two-phase schedule). The last partial round is predicated.
template <int U>
__device__ __forceinline__ void spmv_row_cg1(const PcgArgs& a, const float4* __restrict__ rec, int c, int lane,
											 float al, float be, float& a0, float& a1, float& a2)
{
	const int k0 = __ldg(&a.off[c]), k1 = __ldg(&a.off[c + 1]);
	int k = k0;
	int Jn[U];
#pragma unroll
	for (int u = 0; u < U; ++u) Jn[u] = (k + u < k1) ? __ldcs(&a.col[(k + u) * 32 + lane]) : 0;
	for (;;)
	{
		const int nk = min(U, k1 - k);  // the same in every lane
		if (nk <= 0) break;
		int J[U];
#pragma unroll
		for (int u = 0; u < U; ++u) J[u] = Jn[u];
#pragma unroll
		for (int u = 0; u < U; ++u)
			if (k + U + u < k1) Jn[u] = __ldcs(&a.col[(k + U + u) * 32 + lane]);
		float4 R[U], W[U], S[U];
		float v[U][9];
#pragma unroll
		for (int u = 0; u < U; ++u)
			if (u < nk)
			{
				R[u] = rec[3 * J[u]];
				W[u] = rec[3 * J[u] + 1];
				S[u] = rec[3 * J[u] + 2];
				const float* vb = a.val + (size_t)(k + u) * 288 + lane;
#pragma unroll
				for (int m = 0; m < 9; ++m) v[u][m] = __ldcs(vb + 32 * m);
			}
#pragma unroll
		for (int u = 0; u < U; ++u)
			if (u < nk)
			{
				float s0, s1, s2, r0, r1, r2, p0, p1, p2;
				cg1_next(R[u], W[u], S[u], al, be, s0, s1, s2, r0, r1, r2, p0, p1, p2);
				a0 += v[u][0] * p0 + v[u][1] * p1 + v[u][2] * p2;
				a1 += v[u][3] * p0 + v[u][4] * p1 + v[u][5] * p2;
				a2 += v[u][6] * p0 + v[u][7] * p1 + v[u][8] * p2;
			}
		k += U;
	}
}

// kPcgMixed1, after a refresh (and to start): w[row] = sum of A_block * u(J) with u(J) = d(J) r(J),
// r(J) = (float)(r64(J) / s) the neighbour's rescaled true residual. The owner rounds its own r and u
// by the same expressions. One slot at a time, the next slot's column loaded ahead (a few phases a
// solve).
__device__ __forceinline__ void spmv_row_r64(const PcgArgs& a, int c, int lane, double inv, float& a0, float& a1,
											 float& a2)
{
	const int k0 = __ldg(&a.off[c]), k1 = __ldg(&a.off[c + 1]);
	int Jn = (k0 < k1) ? __ldcs(&a.col[k0 * 32 + lane]) : 0;
	for (int k = k0; k < k1; ++k)
	{
		const int J = Jn;
		if (k + 1 < k1) Jn = __ldcs(&a.col[(k + 1) * 32 + lane]);
		float p[3];
#pragma unroll
		for (int j = 0; j < 3; ++j) p[j] = __fmul_rn(a.invd[3 * J + j], __double2float_rn(a.r64[3 * J + j] * inv));
		const float* vb = a.val + (size_t)k * 288 + lane;
		a0 += __ldcs(vb) * p[0] + __ldcs(vb + 32) * p[1] + __ldcs(vb + 64) * p[2];
		a1 += __ldcs(vb + 96) * p[0] + __ldcs(vb + 128) * p[1] + __ldcs(vb + 160) * p[2];
		a2 += __ldcs(vb + 192) * p[0] + __ldcs(vb + 224) * p[1] + __ldcs(vb + 256) * p[2];
	}
}

// Error-free transformations in FP32 (Knuth's TwoSum; the product's rounding error by FMA):
// a + b = s + e and a * b = p + e exactly. The _rn intrinsics keep the compiler from contracting or
// reassociating them.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
	s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// True residual rows of chunk c: r64 = b - A (x_hl + x_delta); returns the lane's |r|^2 share.
// A x is accumulated in double-float arithmetic: per column the solution t + u = (hi + x_delta) + lo
// with t the rounded sum, every product a t split exactly into p + e by FMA, p added to the row's
// high word by TwoSum and the low parts (TwoSum error, product error, a u) into its low word, the
// pair renormalised once a block. Only b - (hi + lo) runs in FP64, once per row. On random rows of up
// to 81 terms with strong cancellation the error stays within 1.4e-14 of sum |a x| (FP64
// accumulation of the same rows: ~1e-14), at about 140 FP32 operations a block against 9 FP64 FMAs,
// which run at 1/64 of the FP32 rate here.
__device__ __forceinline__ double residual_row(const PcgArgs& a, int c, int rs, int lane)
{
	float sh[3] = {0.f, 0.f, 0.f}, sl[3] = {0.f, 0.f, 0.f};
	const int k0 = __ldg(&a.off[c]), k1 = __ldg(&a.off[c + 1]);
	// The next slot's column is loaded one slot ahead, so a slot waits on one gather, not a
	// column load followed by a gather.
	int Jn = (k0 < k1) ? __ldcs(&a.col[k0 * 32 + lane]) : 0;
	for (int k = k0; k < k1; ++k)
	{
		const int J = Jn;
		if (k + 1 < k1) Jn = __ldcs(&a.col[(k + 1) * 32 + lane]);
		const float* vp = a.val + (size_t)k * 288 + lane;
		float t[3], u[3];
#pragma unroll
		for (int j = 0; j < 3; ++j)
		{
			const float2 x = a.xhl[3 * J + j];
			float e;
			two_sum(x.x, a.xd[3 * J + j], t[j], e);
			u[j] = __fadd_rn(e, x.y);
		}
#pragma unroll
		for (int i = 0; i < 3; ++i)
#pragma unroll
			for (int j = 0; j < 3; ++j)
			{
				const float v = __ldcs(vp + 32 * (3 * i + j));
				const float p = __fmul_rn(v, t[j]);
				const float pe = __fmaf_rn(v, t[j], -p);
				float hs, he;
				two_sum(sh[i], p, hs, he);
				sh[i] = hs;
				sl[i] = __fadd_rn(sl[i], __fadd_rn(he, __fmaf_rn(v, u[j], pe)));
			}
		// Renormalise each row's pair once a block, so the low word stays below half an ulp of the
		// high word and its own rounding stays at 2^-48 of the partial sum.
#pragma unroll
		for (int i = 0; i < 3; ++i)
		{
			float hs, hl;
			two_sum(sh[i], sl[i], hs, hl);
			sh[i] = hs;
			sl[i] = hl;
		}
	}
	double rr = 0.0;
#pragma unroll
	for (int i = 0; i < 3; ++i)
	{
		const double ri = a.brs[3 * rs + i] - (double(sh[i]) + double(sl[i]));
		a.r64[3 * rs + i] = ri;
		rr += ri * ri;
	}
	return rr;
}

}  // namespace

template <int kForm>
__global__ void __launch_bounds__(kPcgThreads, kForm == kPcgF64 ? 3 : 4) k_pcg_persistent(PcgArgs a)
{
	constexpr bool kF64 = kForm == kPcgF64;
	constexpr bool kOne = kForm == kPcgMixed1;
	constexpr int kRound = 2;  // records gathered a round by the one-phase SpMV (64 registers)
	extern __shared__ double dsm[];
	const int lane = threadIdx.x & 31;
	const int warp = threadIdx.x >> 5;
	const int nseg = a.nsegs, M = a.maxChunksPerCta, G = gridDim.x, B = blockIdx.x;
	double* sp = dsm;                                      // [kPcgNV][M] chunk partials of this CTA
	int* sc = reinterpret_cast<int*>(dsm + kPcgNV * M);    // segChunk copy (chunk prefix of all segments)
	int* Cp = sc + (nseg + 1);                         // active set: chunk prefix
	int* Wp = Cp + (nseg + 1);                         // active set: weight prefix
	int* segW = Wp + (nseg + 1);                       // per-segment SpMV weight (block columns + 2 per chunk)
	__shared__ int shRange[4];
	__shared__ int shFinished;
	__shared__ int shNext;  // next position of the current phase (for_chunks)
	// Scalars of the segments in this CTA's range for the current phase (cache_segments).
	constexpr int kSegCache = 32;
	__shared__ double cBeta[kSegCache], cAlpha[kSegCache], cS[kSegCache], cRatio[kSegCache];
	__shared__ int cMode[kSegCache];
	__shared__ int cFirst, cCount;
	if (threadIdx.x == 0) shNext = 0;
	for (int i = threadIdx.x; i <= nseg; i += blockDim.x) sc[i] = a.segChunk[i];
	__syncthreads();
	for (int s = threadIdx.x; s < nseg; s += blockDim.x) segW[s] = __ldg(&a.cumW[sc[s + 1]]) - __ldg(&a.cumW[sc[s]]);
	__syncthreads();

	// zp records: float4 pair per row, .x/.y/.z used: [2*rs] = z = invdiag * r, [2*rs + 1] = p.
	float4* zpOld = reinterpret_cast<float4*>(a.pA);
	float4* zpNew = reinterpret_cast<float4*>(a.pB);
	// FP64 form: {z0 z1 | z2 - | p0 p1 | p2 -} per row.
	double2* zOld64 = reinterpret_cast<double2*>(a.zA64);
	double2* zNew64 = reinterpret_cast<double2*>(a.zB64);

	int ph = 0;  // phase id, the same in every CTA; segments finished in phase ph are stamped ph + 1
	auto finish = [&](SegCtl& S) {
		S.done = ph + 1;
		atomicAdd(&a.g->finishedIn[ph & 1], 1);
		atomicAdd(&a.g->finishedSegs, 1);
	};
	// All chunks, chunk-count partition (positions are chunk ids).
	SetView all;
	all.Cp = sc;
	all.Wp = nullptr;
	all.n = a.nchunks;
	all.tot = a.nchunks;
	all.lo = (int)(((long long)all.n * B + G - 1) / G);
	all.hi = (int)(((long long)all.n * (B + 1) + G - 1) / G);
	SetView actW{}, actC{};  // active set: block-column-weighted and chunk-count partitions (set by rebuild)
	actW.Cp = actC.Cp = Cp;
	actW.Wp = Wp;
	actC.Wp = nullptr;
	// Rebuild the active-set prefixes and this CTA's ranges (segments stamped before phase ph are
	// out). In phase 1 a segment switched to its true residual in the phase before weighs
	// refreshWeight times its block columns. Returns whether any segment was so weighted.
	__shared__ int shWeighted;
	auto rebuild = [&](bool phase1) {
		// Stage every segment's chunk count and weight in Cp[s + 1] / Wp[s + 1] with one round of
		// loads by all threads, then scan them in place in warp 0.
		if (threadIdx.x == 0) shWeighted = 0;
		__syncthreads();
		for (int s = threadIdx.x; s < nseg; s += blockDim.x)
		{
			int c = 0, w = 0;
			const int d = ldi(&a.seg[s].done);
			if (d == 0 || d > ph)
			{
				c = sc[s + 1] - sc[s];
				w = segW[s];
				if (phase1 && ldi(&a.seg[s].refreshAt) == ph - 1)
				{
					w *= a.refreshWeight;
					atomicExch(&shWeighted, 1);
				}
			}
			Cp[s + 1] = c;
			Wp[s + 1] = w;
		}
		__syncthreads();
		if (warp == 0)
		{
			int carryC = 0, carryW = 0;
			if (lane == 0) Cp[0] = Wp[0] = 0;
			for (int base = 0; base < nseg; base += 32)
			{
				const int s = base + lane;
				int c = (s < nseg) ? Cp[s + 1] : 0, w = (s < nseg) ? Wp[s + 1] : 0;
#pragma unroll
				for (int o = 1; o < 32; o <<= 1)
				{
					const int tc = __shfl_up_sync(kFull, c, o), tw = __shfl_up_sync(kFull, w, o);
					if (lane >= o)
					{
						c += tc;
						w += tw;
					}
				}
				if (s < nseg)
				{
					Cp[s + 1] = carryC + c;
					Wp[s + 1] = carryW + w;
				}
				carryC += __shfl_sync(kFull, c, 31);
				carryW += __shfl_sync(kFull, w, 31);
			}
		}
		__syncthreads();
		// This CTA's first position (warp 0) and the next CTA's (warp 1) are independent searches,
		// each a few dependent L2 rounds: run them side by side.
		if (warp < 2)
		{
			const int pos = weighted_start(a, Cp, Wp, sc, nseg, B + warp, G);
			if (lane == 0)
			{
				const long long n = Cp[nseg];
				shRange[warp] = pos;
				shRange[2 + warp] = (int)((n * (B + warp) + G - 1) / G);
			}
		}
		__syncthreads();
		actW.lo = shRange[0];
		actW.hi = shRange[1];
		actC.lo = shRange[2];
		actC.hi = shRange[3];
		if (actW.hi - actW.lo > M || actC.hi - actC.lo > M)
		{
			// Cannot happen with the host's bound on M; clamp so shared memory stays in range.
			if (threadIdx.x == 0) atomicExch(&a.g->err, 2);
			actW.hi = min(actW.hi, actW.lo + M);
			actC.hi = min(actC.hi, actC.lo + M);
		}
		actW.n = actC.n = Cp[nseg];
		actW.tot = Wp[nseg];
		actC.tot = actC.n;
		return shWeighted != 0;
	};
	int finished = 0;        // segments finished before the current phase (same in every CTA)
	bool weighted = false;   // the current partition weighs refreshing segments
	__shared__ int shRefresh;
	// Phase start: count the segments finished (and, before phase 1, switched to a refresh) in the
	// previous phase; rebuild the partition when the active set or the weights change.
	auto phase_start = [&](bool phase1, bool force) {
		if (threadIdx.x == 0)
		{
			shFinished = ldi(&a.g->finishedIn[(ph - 1) & 1]);
			shRefresh = ldi(&a.g->refreshIn[(ph - 1) & 1]);
		}
		__syncthreads();
		const int nf = shFinished;
		finished += nf;
		if (force || nf > 0 || (phase1 && (shRefresh > 0 || weighted))) weighted = rebuild(phase1);
	};
	// Scalars of the segments overlapping this CTA's range of view V, loaded once per phase by all
	// threads (the chunk loops then read shared memory instead of two dependent L2 loads a chunk).
	// They were written before the phase's grid barrier and do not change while the segment's chunks
	// are processed (a segment's reduction completes only after all of its chunks).
	auto cache_segments = [&](const SetView& V) {
		if (threadIdx.x == 0)
		{
			int s0 = 0, cnt = 0;
			if (V.lo < V.hi)
			{
				s0 = seg_of(V.Cp, nseg, V.lo);
				cnt = min(seg_of(V.Cp, nseg, V.hi - 1) - s0 + 1, kSegCache);
			}
			cFirst = s0;
			cCount = cnt;
		}
		__syncthreads();
		for (int i = threadIdx.x; i < cCount; i += blockDim.x)
		{
			const SegCtl* S = &a.seg[cFirst + i];
			double beta;
			int mode;
			load_beta_mode(S, beta, mode);
			const double2 as2 = ldv2(&S->alpha);
			cBeta[i] = beta;
			cMode[i] = mode;
			cAlpha[i] = as2.x;
			cS[i] = as2.y;
			cRatio[i] = ldd(&S->ratio);
		}
		__syncthreads();
	};
	// phase_start and cache_segments for view V in one round of loads: the scalars of the segments in
	// this CTA's range of V as the partition stands are loaded together with the previous phase's
	// finish and refresh counts; only when those call for a new partition is the cache loaded again.
	auto phase_begin = [&](bool phase1, bool force, const SetView& V) {
		if (force)
		{
			phase_start(phase1, true);
			cache_segments(V);
			return;
		}
		if (threadIdx.x == 0)
		{
			int s0 = 0, cnt = 0;
			if (V.lo < V.hi)
			{
				s0 = seg_of(V.Cp, nseg, V.lo);
				cnt = min(seg_of(V.Cp, nseg, V.hi - 1) - s0 + 1, kSegCache);
			}
			cFirst = s0;
			cCount = cnt;
		}
		__syncthreads();
		if (threadIdx.x == kPcgThreads - 32)
		{
			shFinished = ldi(&a.g->finishedIn[(ph - 1) & 1]);
			shRefresh = ldi(&a.g->refreshIn[(ph - 1) & 1]);
		}
		for (int i = threadIdx.x; i < cCount; i += blockDim.x)
		{
			const SegCtl* S = &a.seg[cFirst + i];
			double beta;
			int mode;
			load_beta_mode(S, beta, mode);
			const double2 as2 = ldv2(&S->alpha);
			cBeta[i] = beta;
			cMode[i] = mode;
			cAlpha[i] = as2.x;
			cS[i] = as2.y;
			cRatio[i] = ldd(&S->ratio);
		}
		__syncthreads();
		const int nf = shFinished;
		finished += nf;
		if (nf > 0 || (phase1 && (shRefresh > 0 || weighted)))
		{
			weighted = rebuild(phase1);
			cache_segments(V);
		}
	};
	// {beta, mode, alpha, s, ratio} of segment s: from the phase's cache, else from global memory.
	auto seg_scalars = [&](int s, double& beta, int& mode, double& alpha, double& sv, double& ratio) {
		const int ci = s - cFirst;
		if (ci >= 0 && ci < cCount)
		{
			beta = cBeta[ci];
			mode = cMode[ci];
			alpha = cAlpha[ci];
			sv = cS[ci];
			ratio = cRatio[ci];
			return;
		}
		load_beta_mode(&a.seg[s], beta, mode);
		const double2 as2 = ldv2(&a.seg[s].alpha);
		alpha = as2.x;
		sv = as2.y;
		ratio = ldd(&a.seg[s].ratio);
	};
	// CG iteration cap of segment s.
	auto seg_cap = [&](int s) { return a.segMaxIter ? __ldg(&a.segMaxIter[s]) : a.maxIter; };
	auto barrier = [&]() {
		// Every warp has left the phase's for_chunks (reduce_segments began with __syncthreads);
		// grid_barrier's __syncthreads orders this reset before the next phase's first draw.
		if (threadIdx.x == 0) shNext = 0;
		const bool ok = grid_barrier(a.g, ph, a.barrierTimeoutNs);
		++ph;
		return ok;
	};

	// ---- I1: gather b, invdiag into row space; x = 0; p = 0; |b|^2 per segment.
	for_chunks(all, sc, nseg, &shNext, [&](int slot, int, int c) {
		const int rs = 32 * c + lane;
		const int I = a.perm[rs];
		double bb = 0.0;
		if constexpr (kF64)
		{
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				const double bi = (I >= 0) ? a.b[3 * I + k] : 0.0;
				a.r64[3 * rs + k] = bi;
				a.invd64[3 * rs + k] = (I >= 0) ? a.invdiag64[3 * I + k] : 0.0;
				a.x64[3 * rs + k] = 0.0;
				bb += bi * bi;
			}
			zOld64[4 * rs + 2] = make_double2(0.0, 0.0);
			zOld64[4 * rs + 3] = make_double2(0.0, 0.0);
		}
		else
		{
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				const double bi = (I >= 0) ? a.b[3 * I + k] : 0.0;
				a.brs[3 * rs + k] = bi;
				a.r64[3 * rs + k] = bi;
				a.invd[3 * rs + k] = (I >= 0) ? a.invdiag[3 * I + k] : 0.f;
				a.xhl[3 * rs + k] = make_float2(0.f, 0.f);
				a.xd[3 * rs + k] = 0.f;
				if constexpr (kOne) a.pdir[3 * rs + k] = 0.f;
				bb += bi * bi;
			}
			if constexpr (kOne)
				reinterpret_cast<float4*>(a.pA)[3 * rs + 2] = make_float4(0.f, 0.f, 0.f, 0.f);  // s = A p = 0
			else
				zpOld[2 * rs + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
		}
		bb = warp_sum(bb);
		if (lane == 0) sp[slot] = bb;
	});
	reduce_segments<1>(a, all, sc, sp, [&](int s, const double* tot) {
		SegCtl& S = a.seg[s];
		S.bb = tot[0];
		S.rrTrue = tot[0];
		S.threshold = fmax(a.tol * a.tol * tot[0], DBL_MIN);
		S.s = sqrt(tot[0]);
		S.iter = 0;
		S.updates = 0;
		S.mode = kOne ? 2 : 0;  // kPcgMixed1 starts with the rescale phase (r = b / s, w = A u)
		S.refreshAt = -8;
		S.beta = 0.0;
		S.ratio = 0.0;
		S.converged = (tot[0] == 0.0 || tot[0] < S.threshold) ? 1 : 0;
		S.nonfinite = !isfinite(tot[0]);
		if (S.converged || S.nonfinite) finish(S);
	});
	if (!barrier()) return;

	// ---- Out: x (dof space) = x_hl + x_delta.
	auto write_out = [&]() {
		for_chunks(all, sc, nseg, &shNext, [&](int, int, int c) {
			const int rs = 32 * c + lane;
			const int I = a.perm[rs];
			if (I < 0) return;
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				if constexpr (kF64)
					a.x[3 * I + k] = a.x64[3 * rs + k];
				else
				{
					const float2 xv = a.xhl[3 * rs + k];
					a.x[3 * I + k] = (double(xv.x) + double(xv.y)) + double(a.xd[3 * rs + k]);
				}
			}
		});
	};

	if constexpr (kOne)
	{
		// ---- kPcgMixed1: one grid phase an iteration (Chronopoulos and Gear). Stored per row:
		// record {r_k, d}, {w_k = A u_k, d}, {s_{k-1} = A p_{k-1}, d} (gathered by neighbours, two buffers
		// alternating by phase), p_{k-1} and x_delta (own row only). Scalars alpha_k, beta_k per segment.
		// mode 0: p_k = u_k + beta p_{k-1}, s_k = w_k + beta s_{k-1}, x += alpha p_k, r_{k+1} = r_k - alpha s_k,
		//         u_{k+1} = d r_{k+1}, w_{k+1} = A u_{k+1} (u' of gathered rows formed on the fly);
		//         partials r.u, w.u, |r|^2; then beta = g' / g, alpha = g' / (w.u - beta g' / alpha).
		// mode 1: r64 = b - A (x_hl + x_delta) in double-float (the record's s carried to the other buffer).
		// mode 2: fold x, r = r64 / s, u = d r, w = A u, p and s scaled by the residual's rescale; partials as
		//         mode 0; beta from the last r.u before the refresh (rescaled), alpha as mode 0. Also the
		//         first phase (no refresh yet: beta = 0, alpha = r.u / w.u).
		float4* recOld = reinterpret_cast<float4*>(a.pA);
		float4* recNew = reinterpret_cast<float4*>(a.pB);
		const int maxLoop1 = 3 * a.maxIter + 8;  // a refresh takes two extra phases
		for (int it = 0; it < maxLoop1; ++it)
		{
			phase_begin(true, it == 0, actW);
			if (finished >= nseg) break;
			for_chunks(actW, sc, nseg, &shNext, [&](int slot, int s, int c) {
				const int rs = 32 * c + lane;
				const int d0 = 3 * rs;
				double betaD, alphaD, sD, ratioD;
				int mode;
				seg_scalars(s, betaD, mode, alphaD, sD, ratioD);
				float g = 0.f, dl = 0.f, rr = 0.f;
				double rrTrue = 0.0;
				if (mode == 0)
				{
					const float al = float(alphaD), be = float(betaD), as = float(alphaD * sD);
					float w0 = 0.f, w1 = 0.f, w2 = 0.f;
					spmv_row_cg1<kRound>(a, recOld, c, lane, al, be, w0, w1, w2);
					const float4 R = recOld[d0], W = recOld[d0 + 1], S = recOld[d0 + 2];
					float po[3], xo[3];
#pragma unroll
					for (int i = 0; i < 3; ++i)
					{
						po[i] = __ldcs(&a.pdir[d0 + i]);
						xo[i] = __ldcs(&a.xd[d0 + i]);
					}
					float sn[3], rn[3], un[3];
					cg1_next(R, W, S, al, be, sn[0], sn[1], sn[2], rn[0], rn[1], rn[2], un[0], un[1], un[2]);
					const float d[3] = {R.w, W.w, S.w}, r[3] = {R.x, R.y, R.z}, w[3] = {w0, w1, w2};
#pragma unroll
					for (int i = 0; i < 3; ++i)
					{
						const float pk = __fmaf_rn(be, po[i], __fmul_rn(d[i], r[i]));  // u_k = d r_k as formed last phase
						__stcs(&a.pdir[d0 + i], pk);
						__stcs(&a.xd[d0 + i], __fmaf_rn(as, pk, xo[i]));
						g += rn[i] * un[i];
						dl += w[i] * un[i];
						rr += rn[i] * rn[i];
					}
					recNew[d0] = make_float4(rn[0], rn[1], rn[2], d[0]);
					recNew[d0 + 1] = make_float4(w0, w1, w2, d[1]);
					recNew[d0 + 2] = make_float4(sn[0], sn[1], sn[2], d[2]);
				}
				else if (mode == 1)
				{
					rrTrue = residual_row(a, c, rs, lane);
					recNew[d0 + 2] = recOld[d0 + 2];  // s, read by the rescale phase from the other buffer
				}
				else
				{
					const double inv = 1.0 / sD;
					const float ratio = float(ratioD);
					float w0 = 0.f, w1 = 0.f, w2 = 0.f;
					spmv_row_r64(a, c, lane, inv, w0, w1, w2);
					const float4 So = recOld[d0 + 2];
					float2 xo[3];
					float xv[3], po[3], d[3];
					double rv[3];
#pragma unroll
					for (int i = 0; i < 3; ++i)
					{
						xo[i] = a.xhl[d0 + i];
						xv[i] = __ldcs(&a.xd[d0 + i]);
						po[i] = __ldcs(&a.pdir[d0 + i]);
						rv[i] = a.r64[d0 + i];
						d[i] = a.invd[d0 + i];
					}
					const float so[3] = {So.x, So.y, So.z}, w[3] = {w0, w1, w2};
					float r[3], sn[3];
#pragma unroll
					for (int i = 0; i < 3; ++i)
					{
						// Fold x_delta into the float pair: TwoSum, then renormalise.
						float hs, he, h2, l2;
						two_sum(xo[i].x, xv[i], hs, he);
						two_sum(hs, __fadd_rn(he, xo[i].y), h2, l2);
						a.xhl[d0 + i] = make_float2(h2, l2);
						__stcs(&a.xd[d0 + i], 0.f);
						__stcs(&a.pdir[d0 + i], __fmul_rn(po[i], ratio));
						sn[i] = __fmul_rn(so[i], ratio);
						r[i] = __double2float_rn(rv[i] * inv);
						const float u = __fmul_rn(d[i], r[i]);
						g += r[i] * u;
						dl += w[i] * u;
						rr += r[i] * r[i];
					}
					recNew[d0] = make_float4(r[0], r[1], r[2], d[0]);
					recNew[d0 + 1] = make_float4(w0, w1, w2, d[1]);
					recNew[d0 + 2] = make_float4(sn[0], sn[1], sn[2], d[2]);
				}
				if (mode == 1)
				{
					rrTrue = warp_sum(rrTrue);
					if (lane == 0)
					{
						sp[slot] = rrTrue;
						sp[M + slot] = 0.0;
						sp[2 * M + slot] = 0.0;
					}
				}
				else
				{
					g = warp_sum(g);
					dl = warp_sum(dl);
					rr = warp_sum(rr);
					if (lane == 0)
					{
						sp[slot] = g;
						sp[M + slot] = dl;
						sp[2 * M + slot] = rr;
					}
				}
			});
			reduce_segments<3>(a, actW, sc, sp, [&](int s, const double* tot) {
				SegCtl& S = a.seg[s];
				if (S.mode == 1)
				{
					S.rrTrue = tot[0];
					S.updates += 1;
					if (tot[0] < S.threshold)
					{
						S.converged = 1;  // like Eigen, the converging iteration is not counted
						finish(S);
					}
					else if (!isfinite(tot[0]) || S.iter + 1 >= seg_cap(s))
					{
						S.converged = 0;
						S.nonfinite = !isfinite(tot[0]);
						S.iter += 1;
						finish(S);
					}
					else
					{
						const double sNew = sqrt(tot[0]);
						S.ratio = S.s / sNew;
						S.s = sNew;
						S.mode = 2;
					}
					return;
				}
				const double gN = tot[0], dN = tot[1], rr = tot[2];
				S.rr32 = rr;
				if (S.mode == 2)
				{
					double beta = 0.0, alpha;
					if (S.updates == 0)
						alpha = gN / dN;
					else
					{
						beta = gN / (S.rzPend * S.ratio * S.ratio);
						alpha = gN / (dN - beta * gN / S.alpha);
					}
					S.rrLast = rr;
					if (!isfinite(rr) || !isfinite(alpha))
					{
						S.converged = 0;
						S.nonfinite = 1;
						finish(S);
						return;
					}
					S.beta = beta;
					S.alpha = alpha;
					S.rz = gN;
					if (S.updates > 0) S.iter += 1;
					S.mode = 0;
					return;
				}
				if (!isfinite(rr))
				{
					S.converged = 0;
					S.nonfinite = 1;
					finish(S);
				}
				else if (S.s * S.s * rr < S.threshold || rr < a.drop * S.rrLast || S.iter + 1 >= seg_cap(s))
				{
					S.mode = 1;  // true residual of x_{k+1} next
					S.refreshAt = ph;
					S.rzPend = S.rz;
					atomicAdd(&a.g->refreshIn[ph & 1], 1);
				}
				else
				{
					const double beta = gN / S.rz;
					const double alpha = gN / (dN - beta * gN / S.alpha);
					if (!isfinite(alpha))
					{
						S.converged = 0;
						S.nonfinite = 1;
						finish(S);
						return;
					}
					S.beta = beta;
					S.alpha = alpha;
					S.rz = gN;
					S.iter += 1;
				}
			});
			if (!barrier()) return;
			float4* t = recOld;
			recOld = recNew;
			recNew = t;
		}
		write_out();
		return;
	}

	// ---- I2: r = b / s (FP32), z = invdiag r, rz, |r|^2. FP64 form: z = invdiag r, rz (r = b).
	phase_start(false, true);
	for_chunks(actC, sc, nseg, &shNext, [&](int slot, int s, int c) {
		const int rs = 32 * c + lane;
		if constexpr (kF64)
		{
			double z[3], rz = 0.0;
#pragma unroll
			for (int k = 0; k < 3; ++k)
			{
				const double ri = a.r64[3 * rs + k];
				z[k] = a.invd64[3 * rs + k] * ri;
				rz += ri * z[k];
			}
			zOld64[4 * rs] = make_double2(z[0], z[1]);
			zOld64[4 * rs + 1] = make_double2(z[2], 0.0);
			rz = warp_sum(rz);
			if (lane == 0)
			{
				sp[slot] = rz;
				sp[M + slot] = 0.0;
			}
			return;
		}
		const double inv = 1.0 / ldd(&a.seg[s].s);
		float rz = 0.f, rr = 0.f, z[3];
#pragma unroll
		for (int k = 0; k < 3; ++k)
		{
			const float ri = float(a.brs[3 * rs + k] * inv);
			a.r[3 * rs + k] = ri;
			z[k] = a.invd[3 * rs + k] * ri;
			rz += ri * z[k];
			rr += ri * ri;
		}
		zpOld[2 * rs] = make_float4(z[0], z[1], z[2], 0.f);
		rz = warp_sum(rz);
		rr = warp_sum(rr);
		if (lane == 0)
		{
			sp[slot] = rz;
			sp[M + slot] = rr;
		}
	});
	reduce_segments<2>(a, actC, sc, sp, [&](int s, const double* tot) {
		a.seg[s].rz = tot[0];
		a.seg[s].rr32 = tot[1];
		a.seg[s].rrLast = tot[1];
	});
	if (!barrier()) return;

	const int maxLoop = 2 * a.maxIter + 8;  // a refresh takes one extra iteration slot
	for (int it = 0; it < maxLoop; ++it)
	{
		// ---- Phase 1. mode 0: p_new = z + beta p_old (own rows, and on the fly for gathered rows);
		// q = A p_new; pq. mode 1: r64 = b - A (x_hl + x_delta), accumulated in double-float.
		phase_begin(true, false, actW);
		if (finished >= nseg) break;
		for_chunks(actW, sc, nseg, &shNext, [&](int slot, int s, int c) {
			const int rs = 32 * c + lane;
			double part, betaD, alphaU, sU, ratioU;
			int mode;
			seg_scalars(s, betaD, mode, alphaU, sU, ratioU);
			if constexpr (kF64)
			{
				double a0 = 0.0, a1 = 0.0, a2 = 0.0;
				spmv_row_zp64(a, zOld64, c, lane, betaD, a0, a1, a2);
				const double2 z01 = zOld64[4 * rs], z2 = zOld64[4 * rs + 1], p01 = zOld64[4 * rs + 2],
							  p2 = zOld64[4 * rs + 3];
				const double n0 = z01.x + betaD * p01.x, n1 = z01.y + betaD * p01.y, n2 = z2.x + betaD * p2.x;
				zNew64[4 * rs + 2] = make_double2(n0, n1);
				zNew64[4 * rs + 3] = make_double2(n2, 0.0);
				__stcs(&a.q64[3 * rs], a0);
				__stcs(&a.q64[3 * rs + 1], a1);
				__stcs(&a.q64[3 * rs + 2], a2);
				part = warp_sum(n0 * a0 + n1 * a1 + n2 * a2);
			}
			else if (mode == 0)
			{
				const float beta = float(betaD);
				float a0 = 0.f, a1 = 0.f, a2 = 0.f;
				spmv_row_zp(a, zpOld, c, lane, beta, a0, a1, a2);
				const float4 zi = zpOld[2 * rs], pi = zpOld[2 * rs + 1];
				const float4 pn = make_float4(zi.x + beta * pi.x, zi.y + beta * pi.y, zi.z + beta * pi.z, 0.f);
				zpNew[2 * rs + 1] = pn;
				__stcs(&a.q[3 * rs], a0);
				__stcs(&a.q[3 * rs + 1], a1);
				__stcs(&a.q[3 * rs + 2], a2);
				part = warp_sum(pn.x * a0 + pn.y * a1 + pn.z * a2);
			}
			else
				part = warp_sum(residual_row(a, c, rs, lane));
			if (lane == 0) sp[slot] = part;
		});
		reduce_segments<1>(a, actW, sc, sp, [&](int s, const double* tot) {
			SegCtl& S = a.seg[s];
			if (S.mode == 0)
			{
				S.pq = tot[0];
				S.alpha = S.rz / tot[0];
				return;
			}
			S.rrTrue = tot[0];
			S.updates += 1;
			if (tot[0] < S.threshold)
			{
				S.converged = 1;  // like Eigen, the converging iteration is not counted
				finish(S);
			}
			else if (!isfinite(tot[0]) || S.iter + 1 >= seg_cap(s))
			{
				S.converged = 0;
				S.nonfinite = !isfinite(tot[0]);
				S.iter += 1;
				finish(S);
			}
			else
			{
				const double sNew = sqrt(tot[0]);
				S.ratio = S.s / sNew;
				S.s = sNew;
				S.mode = 2;
			}
		});
		if (!barrier()) return;

		// ---- Phase 2. mode 0: x_delta += alpha s p, r -= alpha q, z = invdiag r; |r|^2, r.z; decide
		// on a refresh. mode 2: fold x, r = r64 / s, z = invdiag r, p *= ratio; |r|^2, r.z.
		phase_begin(false, false, actC);
		for_chunks(actC, sc, nseg, &shNext, [&](int slot, int s, int c) {
			const int rs = 32 * c + lane;
			float s0 = 0.f, s1 = 0.f, z[3];
			double betaD, alphaD, sD, ratioD;
			int mode;
			seg_scalars(s, betaD, mode, alphaD, sD, ratioD);
			if constexpr (kF64)
			{
				// x += alpha p, r -= alpha q, z = invdiag r; |r|^2, r.z (all loads first).
				const int d0 = 3 * rs;
				double iv[3], xv[3], rv[3], qv[3], zz[3];
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					iv[i] = __ldcs(&a.invd64[d0 + i]);
					xv[i] = __ldcs(&a.x64[d0 + i]);
					rv[i] = __ldcs(&a.r64[d0 + i]);
					qv[i] = __ldcs(&a.q64[d0 + i]);
				}
				const double2 p01 = zNew64[4 * rs + 2], p2 = zNew64[4 * rs + 3];
				const double pv[3] = {p01.x, p01.y, p2.x};
				double t0 = 0.0, t1 = 0.0;
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					const double ri = rv[i] - alphaD * qv[i];
					__stcs(&a.x64[d0 + i], xv[i] + alphaD * pv[i]);
					__stcs(&a.r64[d0 + i], ri);
					zz[i] = iv[i] * ri;
					t0 += ri * ri;
					t1 += ri * zz[i];
				}
				zNew64[4 * rs] = make_double2(zz[0], zz[1]);
				zNew64[4 * rs + 1] = make_double2(zz[2], 0.0);
				t0 = warp_sum(t0);
				t1 = warp_sum(t1);
				if (lane == 0)
				{
					sp[slot] = t0;
					sp[M + slot] = t1;
				}
				return;
			}
			// Row-local vectors, touched once a phase: streaming hint (L2 keeps the z/p records). All
			// of a row's loads are issued before its first store (the compiler cannot move a load
			// of one array past a store to another), so a chunk waits on one round of latency.
			const int d0 = 3 * rs;
			float iv[3];
#pragma unroll
			for (int i = 0; i < 3; ++i) iv[i] = __ldcs(&a.invd[d0 + i]);
			if (mode == 0)
			{
				const float alpha = float(alphaD);
				const float as = float(alphaD * sD);
				float xv[3], rv[3], qv[3];
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					xv[i] = __ldcs(&a.xd[d0 + i]);
					rv[i] = __ldcs(&a.r[d0 + i]);
					qv[i] = __ldcs(&a.q[d0 + i]);
				}
				const float4 pn = zpNew[2 * rs + 1];
				const float pv[3] = {pn.x, pn.y, pn.z};
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					const float ri = rv[i] - alpha * qv[i];
					__stcs(&a.xd[d0 + i], xv[i] + as * pv[i]);
					__stcs(&a.r[d0 + i], ri);
					z[i] = iv[i] * ri;
					s0 += ri * ri;
					s1 += ri * z[i];
				}
			}
			else
			{
				const double inv = 1.0 / sD;
				const float ratio = float(ratioD);
				float2 xo[3];
				float xv[3];
				double rv[3];
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					xo[i] = a.xhl[d0 + i];
					xv[i] = __ldcs(&a.xd[d0 + i]);
					rv[i] = __ldcs(&a.r64[d0 + i]);
				}
				const float4 po = zpOld[2 * rs + 1];
#pragma unroll
				for (int i = 0; i < 3; ++i)
				{
					// Fold x_delta into the float pair: TwoSum, then renormalise.
					float hs, he, h2, l2;
					two_sum(xo[i].x, xv[i], hs, he);
					two_sum(hs, __fadd_rn(he, xo[i].y), h2, l2);
					a.xhl[d0 + i] = make_float2(h2, l2);
					__stcs(&a.xd[d0 + i], 0.f);
					const float ri = float(rv[i] * inv);
					__stcs(&a.r[d0 + i], ri);
					z[i] = iv[i] * ri;
					s0 += ri * ri;
					s1 += ri * z[i];
				}
				zpNew[2 * rs + 1] = make_float4(po.x * ratio, po.y * ratio, po.z * ratio, 0.f);
			}
			zpNew[2 * rs] = make_float4(z[0], z[1], z[2], 0.f);
			s0 = warp_sum(s0);
			s1 = warp_sum(s1);
			if (lane == 0)
			{
				sp[slot] = s0;
				sp[M + slot] = s1;
			}
		});
		reduce_segments<2>(a, actC, sc, sp, [&](int s, const double* tot) {
			SegCtl& S = a.seg[s];
			if constexpr (kF64)
			{
				// Eigen's ConjugateGradient: stop on |r|^2 < threshold (the converging iteration is not
				// counted), else beta, and stop at the iteration cap.
				S.rr32 = tot[0];
				S.rrTrue = tot[0];
				if (!isfinite(tot[0]) || !isfinite(S.alpha))
				{
					S.converged = 0;
					S.nonfinite = 1;
					finish(S);
				}
				else if (tot[0] < S.threshold)
				{
					S.converged = 1;
					finish(S);
				}
				else
				{
					S.beta = tot[1] / S.rz;
					S.rz = tot[1];
					S.iter += 1;
					if (S.iter >= seg_cap(s))
					{
						S.converged = 0;
						finish(S);
					}
				}
				return;
			}
			if (S.mode == 2)
			{
				S.beta = tot[1] / (S.rzPend * S.ratio * S.ratio);
				S.rz = tot[1];
				S.rr32 = tot[0];
				S.rrLast = tot[0];
				S.iter += 1;
				S.mode = 0;
				return;
			}
			S.rr32 = tot[0];
			if (!isfinite(tot[0]) || !isfinite(S.alpha))
			{
				S.converged = 0;
				S.nonfinite = 1;
				finish(S);
			}
			else if (S.s * S.s * tot[0] < S.threshold || tot[0] < a.drop * S.rrLast || S.iter + 1 >= seg_cap(s))
			{
				S.mode = 1;  // true residual before the next direction
				S.refreshAt = ph;
				S.rzPend = S.rz;
				atomicAdd(&a.g->refreshIn[ph & 1], 1);
			}
			else
			{
				const double rzOld = S.rz;
				S.rz = tot[1];
				S.beta = tot[1] / rzOld;
				S.iter += 1;
			}
		});
		if (!barrier()) return;
		float4* t = zpOld;
		zpOld = zpNew;
		zpNew = t;
		double2* t64 = zOld64;
		zOld64 = zNew64;
		zNew64 = t64;
	}
	write_out();
}

template __global__ void k_pcg_persistent<kPcgMixed2>(PcgArgs a);
template __global__ void k_pcg_persistent<kPcgF64>(PcgArgs a);
template __global__ void k_pcg_persistent<kPcgMixed1>(PcgArgs a);

namespace {
using PcgKernel = void (*)(PcgArgs);
PcgKernel pcg_kernel(int form)
{
	switch (form)
	{
	case kPcgF64: return k_pcg_persistent<kPcgF64>;
	case kPcgMixed1: return k_pcg_persistent<kPcgMixed1>;
	default: return k_pcg_persistent<kPcgMixed2>;
	}
}
}  // namespace

cudaError_t pcg_set_max_dynamic_smem(int form, int bytes)
{
	return cudaFuncSetAttribute(pcg_kernel(form), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

cudaError_t pcg_occupancy(int form, int* ctasPerSM, size_t smem)
{
	return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctasPerSM, pcg_kernel(form), kPcgThreads, smem);
}

cudaError_t pcg_launch(int form, const cudaLaunchConfig_t& cfg, const PcgArgs& a)
{
	return cudaLaunchKernelEx(&cfg, pcg_kernel(form), a);
}

namespace {

__global__ void k_step_accumulate(const SegCtl* __restrict__ seg, int nseg, const int* __restrict__ ctlNonfinite,
								  const int* __restrict__ pcgErr, double* __restrict__ acc)
{
	for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nseg; k += gridDim.x * blockDim.x)
	{
		const SegCtl& c = seg[k];
		const double res = c.bb > 0 ? sqrt(c.rrTrue / c.bb) : 0.0;
		acc[4 * k] += c.iter;
		acc[4 * k + 1] += c.updates;
		acc[4 * k + 2] = fmin(acc[4 * k + 2], (double)c.converged);
		acc[4 * k + 3] = fmax(acc[4 * k + 3], res);
	}
	if (blockIdx.x == 0 && threadIdx.x == 0)
	{
		if (*ctlNonfinite) acc[4 * nseg] = 1.0;
		if (*pcgErr) acc[4 * nseg + 1] = 1.0;
	}
}

}  // namespace

__global__ void __launch_bounds__(32) k_barrier_selftest(PcgGlobal* g, int phases, int stall, long long timeoutNs,
														 long long* out)
{
	// Block 0 adds gridDim.x before its own first arrival (same thread, same address: in order).
	// Arrivals before the add come from the other gridDim.x - 1 blocks and return at most
	// gridDim.x - 2; arrivals after it return at least gridDim.x. None returns gridDim.x - 1, so no
	// block releases the barrier and every wait runs out.
	if (stall && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&g->barCount, gridDim.x);
	const unsigned long long t0 = global_ns();
	int passed = 0;
	for (int ph = 0; ph < phases; ++ph)
	{
		if (!grid_barrier(g, ph, timeoutNs)) break;
		++passed;
	}
	if (threadIdx.x == 0)
	{
		out[2 * blockIdx.x] = passed;
		out[2 * blockIdx.x + 1] = (long long)(global_ns() - t0);
	}
}

void launch_step_accumulate(const SegCtl* seg, int nseg, const int* ctlNonfinite, const int* pcgErr, double* acc,
							cudaStream_t s)
{
	k_step_accumulate<<<(nseg + 127) / 128, 128, 0, s>>>(seg, nseg, ctlNonfinite, pcgErr, acc);
}

}  // namespace gbfem
