// garm_noalloc.cu — WENO5 reinitialisation of a device-resident field that
// allocates nothing.
//
// Who needs it: code that may not call cudaMalloc at all — a plug-in running
// inside a host application that owns every byte of device memory (a renderer or
// engine with a fixed memory budget), or a real-time loop that must not take the
// implicit device synchronisation cudaMalloc/cudaFree can cause.  Such a caller
// passes its own device field; the two TVD-RK3 stage planes the scheme needs live
// in the fixed array below instead of in per-call allocations.
//
// The array is a file-scope __device__ variable, so every GPU that loads this
// library holds GARM_NOALLOC_MAX_CELLS * 2 doubles (8 MiB) until the process exits.
// Host code cannot use the array's name as a device address (in host code it is
// only a stand-in symbol), so the address is fetched with cudaGetSymbolAddress,
// once per device, with that device current, on the first call made there.
//
// Nothing here blocks the host either: the launch plan is the one already cached
// or pinned for the grid shape (garm_reinit_plan_set, or an earlier tuned call
// through another entry point), else the default column plan.  This entry point
// never runs the autotuner, whose candidate timings synchronise the stream.
#include "garm_internal.h"

#include <mutex>

namespace {

constexpr int64_t kMaxCells = GARM_NOALLOC_MAX_CELLS;
constexpr int kMaxDevices = 64;

// Two stage planes of up to kMaxCells doubles each.  Every call overwrites a plane
// completely before reading it, so nothing has to be cleared between calls.
static __device__ __align__(256) double g_reinitScratch[2 * kMaxCells];

std::mutex g_scratchMutex;
double *g_scratchAddr[kMaxDevices] = {};

// Device address of the scratch array on the current device (looked up once).
garm_status scratchOnCurrentDevice(double **out) {
	int dev = -1;
	if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return GARM_CUDA_ERROR; }
	if (dev < 0 || dev >= kMaxDevices) return GARM_UNSUPPORTED;
	std::lock_guard<std::mutex> lock(g_scratchMutex);
	if (!g_scratchAddr[dev]) {
		void *p = nullptr;
		const cudaError_t e = cudaGetSymbolAddress(&p, g_reinitScratch);
		if (e != cudaSuccess || !p) { cudaGetLastError(); return GARM_CUDA_ERROR; }
		g_scratchAddr[dev] = static_cast<double *>(p);
	}
	*out = g_scratchAddr[dev];
	return GARM_OK;
}

}  // namespace

extern "C" garm_status garm_reinit_device_noalloc(int dim, const int *size, double spacing, double *phi, int iters, double cfl, void *stream) {
	if ((dim != 2 && dim != 3) || !size || !phi || !(spacing > 0) || iters < 0 || !(cfl > 0)) return GARM_INVALID;
	int64_t n = 1;
	for (int a = 0; a < dim; a++) {
		if (size[a] <= 0) return GARM_INVALID;
		n *= size[a];
		if (n > kMaxCells) return GARM_INVALID;  // larger than the fixed scratch
	}
	// phi must be memory of the current device (or managed memory): a host pointer
	// handed over by mistake would be dereferenced by the stencil kernels
	cudaPointerAttributes attr{};
	if (cudaPointerGetAttributes(&attr, phi) != cudaSuccess) { cudaGetLastError(); return GARM_INVALID; }
	int dev = -1;
	if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return GARM_CUDA_ERROR; }
	if (attr.type == cudaMemoryTypeDevice ? attr.device != dev : attr.type != cudaMemoryTypeManaged) return GARM_INVALID;
	double *scratch = nullptr;
	GARM_TRY(scratchOnCurrentDevice(&scratch));
	const cudaStream_t st = static_cast<cudaStream_t>(stream);
	// FP64 never takes the tiled form, the only one with an error flag; tune = false keeps
	// the autotuner (and its stream synchronisations) off this path
	if (dim == 2) return garm::reinitRaw<2, double>(st, size, spacing, phi, scratch, scratch + n, iters, cfl, nullptr, false);
	return garm::reinitRaw<3, double>(st, size, spacing, phi, scratch, scratch + n, iters, cfl, nullptr, false);
}
