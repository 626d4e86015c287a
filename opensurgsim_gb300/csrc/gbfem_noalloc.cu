// gbfem_noalloc.cu -- a Jacobi-PCG solve that allocates no device or pinned memory.
//
// Every scratch buffer the solve needs (preconditioner, residual, search direction, product,
// reduction partials, control block) lives in one file-scope device array of fixed size, so a
// call makes no cudaMalloc/cudaFree/cudaMallocHost or allocating library call. The array exists on
// every GPU that loads this library, for the life of the process. All calls share it: calls that
// overlap on the GPU (two host threads, or two streams, on the same device) race on it and must be
// serialised by the caller. The control block is cleared at the start of every call; the other
// buffers are fully written before they are read.

#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gbfem.h"
#include "gbfem_internal.h"

namespace gbfem {
namespace noalloc {
constexpr int kMaxDofs = GBFEM_NOALLOC_MAX_DOFS;
constexpr int kGrid = 152 * 8;  // blocks of the dof-wise kernels (and reduction partial slots)
// Layout inside the scratch array (all offsets multiples of 256 bytes).
constexpr size_t kVecBytes = ((size_t)kMaxDofs * sizeof(double) + 255) / 256 * 256;
constexpr size_t kPartBytes = ((size_t)partial_slots(kGrid) * sizeof(double) + 255) / 256 * 256;
constexpr size_t kCtlBytes = (sizeof(CgCtl) + 255) / 256 * 256;
constexpr size_t kScratchBytes = 4 * kVecBytes + kPartBytes + kCtlBytes;
}  // namespace noalloc
void set_global_error(const std::string& msg);  // message returned by gbfem_last_error(NULL, ...)
}  // namespace gbfem

// The scratch array: about 8.5 MB of device memory on every GPU that loads the library.
static __device__ __align__(256) unsigned char g_noallocScratch[gbfem::noalloc::kScratchBytes];

namespace gbfem {
namespace {
using namespace noalloc;
constexpr int kNoAllocMaxDofs = kMaxDofs;
constexpr int kNoAllocGrid = kGrid;

// Host-side copy of the scratch array's device address, per device. The array's name in host
// code is only a host stand-in; its device address comes from cudaGetSymbolAddress, taken once per
// device with that device current.
constexpr int kMaxDevices = 64;
unsigned char* g_scratchAddr[kMaxDevices] = {};
std::mutex g_scratchMutex;


__global__ void k_noalloc_invdiag(int n, const int* __restrict__ rowptr, const int* __restrict__ col,
								  const double* __restrict__ val, double* __restrict__ invdiag)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
	{
		double d = 0.0;
		for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
			if (col[k] == i) d = val[k];
		invdiag[i] = (d != 0.0) ? 1.0 / d : 1.0;  // DiagonalPreconditioner
	}
}

gbfem_status scratch_for_current_device(unsigned char** out)
{
	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return GBFEM_CUDA_ERROR;
	if (dev < 0 || dev >= kMaxDevices)
	{
		set_global_error("device ordinal out of range");
		return GBFEM_INVALID_ARG;
	}
	std::lock_guard<std::mutex> lock(g_scratchMutex);
	if (!g_scratchAddr[dev])
	{
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noallocScratch);
		if (e != cudaSuccess || !p)
		{
			set_global_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
			return GBFEM_CUDA_ERROR;
		}
		g_scratchAddr[dev] = static_cast<unsigned char*>(p);
	}
	*out = g_scratchAddr[dev];
	return GBFEM_OK;
}

}  // namespace
}  // namespace gbfem

using namespace gbfem;

extern "C" gbfem_status gbfem_cg_solve_noalloc(int32_t n, const int32_t* rowptr, const int32_t* col,
											   const double* values, const double* b, double* x, double tolerance,
											   int32_t max_iterations, void* stream, int32_t* iterations,
											   double* relative_residual)
{
	if (n <= 0 || !rowptr || !col || !values || !b || !x || !(tolerance >= 0.0))
	{
		set_global_error("gbfem_cg_solve_noalloc: invalid argument");
		return GBFEM_INVALID_ARG;
	}
	if (n > kNoAllocMaxDofs)
	{
		set_global_error("gbfem_cg_solve_noalloc: n = " + std::to_string(n) +
						 " exceeds the fixed scratch capacity of " + std::to_string(kNoAllocMaxDofs) +
						 " dofs (GBFEM_NOALLOC_MAX_DOFS)");
		return GBFEM_INVALID_ARG;
	}
	unsigned char* base = nullptr;
	gbfem_status st = scratch_for_current_device(&base);
	if (st != GBFEM_OK) return st;
	double* invdiag = reinterpret_cast<double*>(base);
	double* r = reinterpret_cast<double*>(base + kVecBytes);
	double* p = reinterpret_cast<double*>(base + 2 * kVecBytes);
	double* q = reinterpret_cast<double*>(base + 3 * kVecBytes);
	double* part = reinterpret_cast<double*>(base + 4 * kVecBytes);
	CgCtl* ctl = reinterpret_cast<CgCtl*>(base + 4 * kVecBytes + kPartBytes);

	Launch L;
	L.stream = static_cast<cudaStream_t>(stream);
	L.vecGrid = std::max(1, std::min((n + 255) / 256, kNoAllocGrid));
	const int maxIter = max_iterations > 0 ? max_iterations : 2 * n;
	auto ok = [](cudaError_t e) { return e == cudaSuccess; };
	if (!ok(cudaMemsetAsync(ctl, 0, sizeof(CgCtl), L.stream))) return GBFEM_CUDA_ERROR;
	k_noalloc_invdiag<<<L.vecGrid, 256, 0, L.stream>>>(n, rowptr, col, values, invdiag);
	MatCsr A{n, rowptr, col, values};
	launch_cg_init(n, b, invdiag, x, r, p, ctl, part, tolerance, maxIter, L);
	CgCtl h;  // pageable host copy of the control block (no pinned allocation)
	long long launched = 0;
	int chunk = 4;
	for (;;)
	{
		for (int k = 0; k < chunk; ++k)
		{
			launch_cg_spmv_csr(A, p, q, ctl, part, L);
			launch_cg_update(n, invdiag, p, q, x, r, ctl, part, L);
			launch_cg_pupdate(n, invdiag, r, p, ctl, L);
		}
		launched += chunk;
		if (!ok(cudaMemcpyAsync(&h, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, L.stream)) ||
			!ok(cudaStreamSynchronize(L.stream)))
		{
			set_global_error(cudaGetErrorString(cudaGetLastError()));
			return GBFEM_CUDA_ERROR;
		}
		if (h.done) break;
		if (launched > (long long)maxIter + 64)
		{
			set_global_error("CG control block did not finish");
			return GBFEM_CUDA_ERROR;
		}
		chunk = std::min(chunk * 2, 32);
	}
	if (!ok(cudaGetLastError())) return GBFEM_CUDA_ERROR;
	if (iterations) *iterations = h.iter;
	if (relative_residual) *relative_residual = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
	return h.converged ? GBFEM_OK : GBFEM_CG_MAXITER;
}
