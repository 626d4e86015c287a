// gbfem_pcg.h -- persistent CG over a batch of segments, mixed-precision or FP64 (declarations).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gbfem {

constexpr int kPcgThreads = 256;
constexpr int kPcgChunkWeight = 2;  // per-chunk constant added to the block-column count (SpMV work)

// Forms of the persistent solve (template argument of k_pcg_persistent).
//  kPcgMixed2: FP32 CG in two grid phases an iteration (q = A p with p formed on the fly and p.q;
//              then the row-local x, r, z update with r.z), double-float refreshes;
//  kPcgF64:    plain FP64 CG (Eigen's iteration and stopping rule), the same two phases;
//  kPcgMixed1: FP32 CG in one grid phase an iteration (Chronopoulos and Gear's recurrences: the
//              SpMV w = A u runs on the next preconditioned residual, formed on the fly for gathered
//              rows from their {r, w, s} records, and r.u and w.u come from the same phase), with the
//              same refreshes and stopping rule as kPcgMixed2. Its SpMV gathers two 48-byte records a
//              round (four would spill at 64 registers; at 80 registers and 3 CTAs per SM they measured
//              slower on both the 256-mesh batch and the 1.28M-tet bar, and so did three with a spill).
// Measured on GB300: the one-phase schedule halves the phases; on one 1.28M-tet mesh, whose phases
// wait on latency, its solve takes 17.2 ms against 22.9 ms in two phases, while on the 256-mesh batch,
// whose phases mostly stream the whole batch, it is the slower (53.1 vs 41.3 ms). The autotuner times
// both; without it a handle starts in the schedule its size suggests (kOnePhaseChunksPerSlot).
enum PcgForm : int
{
	kPcgMixed2 = 0,
	kPcgF64 = 1,
	kPcgMixed1 = 2,
};
// Default schedule without autotuning: kPcgMixed1 while the system has at most this many chunks per
// CTA slot of a 4-CTA-per-SM grid, kPcgMixed2 above.
constexpr int kOnePhaseChunksPerSlot = 16;
constexpr int kPcgNV = 3;  // per-chunk partial values a phase can reduce (shared memory, cross-CTA slots)

// Per-segment (per-mesh) CG state, in device memory. Written by the CTA that completes a
// segment's reduction, read by every CTA after the next grid barrier.
struct alignas(16) SegCtl
{
	double beta;            // phase 1 reads {beta, mode, refreshAt} with one 16-byte load
	int mode;               // 0: CG step; 1: FP64 residual next; 2: rescale next
	int refreshAt;          // phase id at which mode 1 was last set
	double alpha, s;        // phase 2 reads {alpha, s} with one 16-byte load; r_true ~= s * r32
	double ratio;
	double bb, threshold;   // |b|^2, tol^2 |b|^2
	double rz, pq;
	double rr32, rrLast;    // |r32|^2 now and right after the last refresh
	double rrTrue;          // |b - A x|^2 at the last refresh
	double rzPend;
	int iter, updates, done, converged;
	int nonfinite;
	unsigned int ticket;
	int pad[2];
};

// Grid-wide control of one persistent launch.
struct PcgGlobal
{
	unsigned int barCount, barGen;
	int finishedSegs;    // total, for diagnostics
	int err;
	int finishedIn[2];   // segments finished in a phase, by phase parity
	int refreshIn[2];    // segments switched to a true-residual refresh in a phase, by phase parity
};

// Weight of a chunk of a segment doing its true residual (phase 1, double-float), relative to an
// FP32 SpMV chunk: a tuning choice (PcgArgs::refreshWeight), at most kRefreshWeightMax. Measured
// best at 2 on the 256-mesh batch (with an FP64 residual it was 6).
constexpr int kRefreshWeightDefault = 2;
constexpr int kRefreshWeightMax = 8;

// Wall-time limit of one grid-barrier wait. A phase of the persistent solve is one pass over at
// most the whole matrix (tens of ms for the largest system that fits in HBM), so a wait this long
// means a block is gone; the solve then ends with PcgGlobal::err set.
constexpr long long kBarrierTimeoutNs = 1000000000LL;

struct PcgArgs
{
	int nchunks, nsegs, maxIter, maxChunksPerCta;
	int refreshWeight, pad;
	double tol, drop;
	long long barrierTimeoutNs;  // wall time a block waits at a grid barrier before it reports an error
	// SELL-32 matrix in row space (column = neighbour row position), FP32 values
	const int* off;        // nchunks + 1
	const int* col;
	const float* val;
	const int* perm;       // row position -> node id, -1 for padding rows
	const int* segChunk;   // nsegs + 1: first chunk of each segment (segments own contiguous chunks)
	const int* segMaxIter; // nsegs: per-segment CG iteration cap, or null: maxIter for every segment
	const int* cumW;       // nchunks + 1: prefix of (block columns + kPcgChunkWeight) per chunk
	double* slots;         // 2 * kPcgNV * grid cross-CTA partials: [value k][first/last][cta]
	// in / out (dof space, FP64)
	const double* b;
	const float* invdiag;
	double* x;
	// row-space work vectors
	double* brs;
	double* r64;
	float2* xhl;           // FP64 part of the solution as an unevaluated float pair hi + lo, 3 per row
	float* xd;
	float* invd;
	float* r;
	float* pA;             // kPcgMixed2: 8 floats per row: z (3), pad, p (3), pad; 32-byte aligned
	float* pB;             // kPcgMixed1: 12 floats per row: {r (3), d0}, {w (3), d1}, {s (3), d2}, d = invdiag
	float* q;
	float* pdir;           // kPcgMixed1: search direction p, 3 floats per row (read by its own row only)
	SegCtl* seg;
	PcgGlobal* g;
	// FP64 form (k_pcg_persistent<true>): plain FP64 CG on the FP64 SELL values, Eigen's iteration and
	// stopping rule for every segment, no refreshes. r in r64, x in x64, b in brs.
	const double* val64;   // FP64 SELL values (same slots as val)
	const double* invdiag64;  // dof space
	double* invd64;        // row space
	double* x64;           // row space
	double* q64;
	double* zA64;          // 8 doubles per row: z (3), pad, p (3), pad; 64-byte aligned
	double* zB64;
};

// Dynamic shared memory of one CTA: the chunk partials, the segment chunk prefix, the active-set
// prefix arrays and the per-segment base weights.
inline size_t pcg_smem_bytes(int nsegs, int maxChunksPerCta)
{
	return kPcgNV * sizeof(double) * (size_t)maxChunksPerCta + 4 * sizeof(int) * (size_t)(nsegs + 1);
}

// kForm: a PcgForm.
template <int kForm>
__global__ void k_pcg_persistent(PcgArgs a);

// Host access to the instantiations (the kernel templates' host stubs are local to their
// translation unit): the dynamic shared memory limit, the co-resident CTAs per SM, and a launch
// with the caller's configuration (grid, block, shared memory, stream, cooperative attribute).
cudaError_t pcg_set_max_dynamic_smem(int form, int bytes);
cudaError_t pcg_occupancy(int form, int* ctasPerSM, size_t smem);
cudaError_t pcg_launch(int form, const cudaLaunchConfig_t& cfg, const PcgArgs& a);

// Self-test of the grid barrier on a PcgGlobal of its own (zeroed by the caller): `phases` barriers
// over a cooperative grid. With `stall` set, the arrival counter starts at gridDim.x, so no block is
// ever the last to arrive and every wait must run out after timeoutNs; each block records in
// out[2 * block] the barriers it passed and in out[2 * block + 1] the wall time it spent, in ns.
__global__ void k_barrier_selftest(PcgGlobal* g, int phases, int stall, long long timeoutNs, long long* out);

// Per-step statistics kept on the device (graph-launched steps): acc[4*s + 0/1/2/3] += iterations,
// += refreshes, min= converged, max= relative residual of segment s; acc[4*nseg] = 1 once a step's
// state was not finite (ctlNonfinite points at the validity kernel's flag), acc[4*nseg + 1] = 1 once
// a solve reported an error (pcgErr).
void launch_step_accumulate(const SegCtl* seg, int nseg, const int* ctlNonfinite, const int* pcgErr, double* acc,
							cudaStream_t s);

}  // namespace gbfem
