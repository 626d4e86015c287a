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

#include <cuda.h>

#include "../../include/gbfem.h"
#include "gbfem_internal.h"

namespace gbfem {
namespace noalloc {
constexpr int kMaxDofs = GBFEM_NOALLOC_MAX_DOFS;
// Upper bound on the grid of the dof-wise kernels, which sizes the reduction partial slots inside
// the fixed scratch array. A call uses 8 blocks per SM of its device, capped at this bound (GB300:
// 152 SMs x 8 = 1216 exactly).
constexpr int kMaxGrid = 1216;
// Layout inside the scratch array (all offsets multiples of 256 bytes).
constexpr size_t kVecBytes = ((size_t)kMaxDofs * sizeof(double) + 255) / 256 * 256;
constexpr size_t kPartBytes = ((size_t)partial_slots(kMaxGrid) * sizeof(double) + 255) / 256 * 256;
constexpr size_t kCtlBytes = (sizeof(CgCtl) + 255) / 256 * 256;
constexpr size_t kFlagBytes = 256;  // input check: first bad row and the kind of fault
constexpr size_t kScratchBytes = 4 * kVecBytes + kPartBytes + kCtlBytes + kFlagBytes;
}  // namespace noalloc
void set_global_error(const std::string& msg);  // message returned by gbfem_last_error(NULL, ...)
}  // namespace gbfem

// The scratch array: about 8.5 MB of device memory on every GPU that loads the library.
static __device__ __align__(256) unsigned char g_noallocScratch[gbfem::noalloc::kScratchBytes];

namespace gbfem {
namespace {
using namespace noalloc;

// Host-side copy of the scratch array's device address and the device's SM count, per device.
// The array's name in host code is only a host stand-in; its device address comes from
// cudaGetSymbolAddress, taken with that device current the first time a call runs in a context of
// the device. The entry is keyed on the context's process-unique id, so a context created after a
// cudaDeviceReset (where the module, and the array, may be loaded at another address) is set up
// again instead of reusing a stale address.
constexpr int kMaxDevices = 64;
struct ScratchEntry
{
	unsigned long long ctxId = 0;
	bool valid = false;
	unsigned char* addr = nullptr;
	int grid = 0;
};
ScratchEntry g_scratch[kMaxDevices];
std::mutex g_scratchMutex;

// Current context id through the driver's cuCtxGetCurrent / cuCtxGetId, looked up at run time
// (the library links only the static CUDA runtime).
bool current_context_id(unsigned long long* id)
{
	static CUresult (*getCurrent)(CUcontext*) = nullptr;
	static CUresult (*getId)(CUcontext, unsigned long long*) = nullptr;
	static std::once_flag once;
	std::call_once(once, [] {
		void* f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
			q == cudaDriverEntryPointSuccess)
			getCurrent = reinterpret_cast<CUresult (*)(CUcontext*)>(f);
		f = nullptr;
		if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
			q == cudaDriverEntryPointSuccess)
			getId = reinterpret_cast<CUresult (*)(CUcontext, unsigned long long*)>(f);
	});
	CUcontext ctx = nullptr;
	if (!getCurrent || !getId || getCurrent(&ctx) != CUDA_SUCCESS || !ctx) return false;
	return getId(ctx, id) == CUDA_SUCCESS;
}

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

// Input check, part 1: rowptr[0] == 0 and rowptr non-decreasing. flag[0] = 2 (rowptr) or 3
// (column, part 2) once a fault is found, flag[1] = lowest bad row (atomicMin).
__global__ void k_noalloc_check_rowptr(int n, const int* __restrict__ rowptr, int* flag)
{
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		if ((i == 0 && rowptr[0] != 0) || rowptr[i + 1] < rowptr[i])
		{
			atomicMax(&flag[0], 2);
			atomicMin(&flag[1], i);
		}
}

// Input check, part 2, only once part 1 found rowptr sound (so every read of col stays inside
// the rowptr[n] entries the caller declares): every column index in [0, n).
__global__ void k_noalloc_check_cols(int n, const int* __restrict__ rowptr, const int* __restrict__ col, int* flag)
{
	if (*(volatile int*)&flag[0] != 0) return;
	for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
		for (int k = rowptr[i]; k < rowptr[i + 1]; ++k)
			if ((unsigned)col[k] >= (unsigned)n)
			{
				atomicMax(&flag[0], 3);
				atomicMin(&flag[1], i);
				break;
			}
}

gbfem_status fail_cuda(const char* what, cudaError_t e)
{
	set_global_error(std::string("gbfem_cg_solve_noalloc: ") + what + ": " + cudaGetErrorString(e));
	return GBFEM_CUDA_ERROR;
}

gbfem_status scratch_for_current_device(unsigned char** out, int* grid)
{
	int dev = -1;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return fail_cuda("cudaGetDevice", e);
	if (dev < 0 || dev >= kMaxDevices)
	{
		set_global_error("gbfem_cg_solve_noalloc: device ordinal out of range");
		return GBFEM_INVALID_ARG;
	}
	unsigned long long ctxId = 0;
	const bool haveId = current_context_id(&ctxId);
	std::lock_guard<std::mutex> lock(g_scratchMutex);
	ScratchEntry& s = g_scratch[dev];
	if (!s.valid || !haveId || s.ctxId != ctxId)
	{
		void* p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noallocScratch);
		if (e != cudaSuccess || !p) return fail_cuda("cudaGetSymbolAddress", e);
		int sms = 0;
		e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
		if (e != cudaSuccess) return fail_cuda("cudaDeviceGetAttribute", e);
		s.addr = static_cast<unsigned char*>(p);
		s.grid = std::max(1, std::min(8 * sms, kMaxGrid));
		s.ctxId = ctxId;
		s.valid = haveId;  // without a context id, look the address up on every call
	}
	*out = s.addr;
	*grid = s.grid;
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
	if (n > kMaxDofs)
	{
		set_global_error("gbfem_cg_solve_noalloc: n = " + std::to_string(n) +
						 " exceeds the fixed scratch capacity of " + std::to_string(kMaxDofs) +
						 " dofs (GBFEM_NOALLOC_MAX_DOFS)");
		return GBFEM_INVALID_ARG;
	}
	unsigned char* base = nullptr;
	int grid = 0;
	gbfem_status st = scratch_for_current_device(&base, &grid);
	if (st != GBFEM_OK) return st;
	double* invdiag = reinterpret_cast<double*>(base);
	double* r = reinterpret_cast<double*>(base + kVecBytes);
	double* p = reinterpret_cast<double*>(base + 2 * kVecBytes);
	double* q = reinterpret_cast<double*>(base + 3 * kVecBytes);
	double* part = reinterpret_cast<double*>(base + 4 * kVecBytes);
	CgCtl* ctl = reinterpret_cast<CgCtl*>(base + 4 * kVecBytes + kPartBytes);
	int* flag = reinterpret_cast<int*>(base + 4 * kVecBytes + kPartBytes + kCtlBytes);

	Launch L;
	L.stream = static_cast<cudaStream_t>(stream);
	L.vecGrid = std::max(1, std::min((n + 255) / 256, grid));
	const int maxIter = max_iterations > 0 ? max_iterations : 2 * n;
	cudaError_t e;
	// The caller's CSR is checked on the device before anything reads through its column indices.
	// The flag starts at {0, 0x7f7f7f7f} (above any row index, for the atomicMin).
	if ((e = cudaMemsetAsync(flag, 0, sizeof(int), L.stream)) != cudaSuccess ||
		(e = cudaMemsetAsync(flag + 1, 0x7f, sizeof(int), L.stream)) != cudaSuccess)
		return fail_cuda("cudaMemsetAsync", e);
	k_noalloc_check_rowptr<<<L.vecGrid, 256, 0, L.stream>>>(n, rowptr, flag);
	k_noalloc_check_cols<<<L.vecGrid, 256, 0, L.stream>>>(n, rowptr, col, flag);
	if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda("input check launch", e);
	int flagHost[2] = {0, 0};
	if ((e = cudaMemcpyAsync(flagHost, flag, sizeof(flagHost), cudaMemcpyDeviceToHost, L.stream)) != cudaSuccess ||
		(e = cudaStreamSynchronize(L.stream)) != cudaSuccess)
		return fail_cuda("input check", e);
	if (flagHost[0] != 0)
	{
		set_global_error(std::string("gbfem_cg_solve_noalloc: ") +
						 (flagHost[0] == 2 ? "rowptr does not start at 0 or decreases" : "column index outside [0, n)") +
						 " at row " + std::to_string(flagHost[1]));
		return GBFEM_INVALID_ARG;
	}
	if ((e = cudaMemsetAsync(ctl, 0, sizeof(CgCtl), L.stream)) != cudaSuccess) return fail_cuda("cudaMemsetAsync", e);
	k_noalloc_invdiag<<<L.vecGrid, 256, 0, L.stream>>>(n, rowptr, col, values, invdiag);
	MatCsr A{n, rowptr, col, values};
	launch_cg_init(n, b, invdiag, x, r, p, ctl, part, tolerance, maxIter, L);
	if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda("launch", e);
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
		if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda("launch", e);
		if ((e = cudaMemcpyAsync(&h, ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, L.stream)) != cudaSuccess ||
			(e = cudaStreamSynchronize(L.stream)) != cudaSuccess)
			return fail_cuda("control block read", e);
		if (h.done) break;
		if (launched > (long long)maxIter + 64)
		{
			set_global_error("gbfem_cg_solve_noalloc: CG control block did not finish");
			return GBFEM_CUDA_ERROR;
		}
		chunk = std::min(chunk * 2, 32);
	}
	if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda("solve", e);
	if (iterations) *iterations = h.iter;
	if (relative_residual) *relative_residual = h.bb > 0 ? std::sqrt(h.rr / h.bb) : 0.0;
	if (!h.converged) set_global_error("gbfem_cg_solve_noalloc: CG stopped at max_iterations");
	return h.converged ? GBFEM_OK : GBFEM_CG_MAXITER;
}
