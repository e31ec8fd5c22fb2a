// garm_selftest.cu — garm_barrier_selftest: the grid barrier of the persistent kernels
// (garm_sync.cuh) on its own, to time a barrier and to exercise its bounded wait.
#include "garm_internal.h"
#include "garm_sync.cuh"

namespace garm {

constexpr int kSelftestBlock = 128;

// `rounds` barriers in a row.  With `neverComplete` every block starts one barrier ahead
// of the counter, so the count it waits for is never reached: each wait runs into the
// time limit, sets the error flag and returns false (the flag nothing else sets).
__global__ void __launch_bounds__(kSelftestBlock) kBarrierSelftest(unsigned *bar, int *err, int rounds, int neverComplete, int *passed) {
	unsigned epoch = neverComplete ? 1u : 0u;
	int r = 0;
	for (; r < rounds; r++)
		if (!gridSync(bar, err, epoch)) break;
	if (blockIdx.x == 0 && threadIdx.x == 0) *passed = r;
}

// FP64 FMA throughput: every thread runs kFmaChains independent dependent chains of
// x = x·a + b, so the FP64 pipe always has ready instructions.  The chains' sum goes to
// `sink` (one store per thread) so that no chain is dead code.
constexpr int kFmaBlock = 256, kFmaChains = 8;

__global__ void __launch_bounds__(kFmaBlock) kFp64Fma(int iters, double a, double b, double *sink) {
	double x[kFmaChains];
#pragma unroll
	for (int c = 0; c < kFmaChains; c++) x[c] = double(threadIdx.x + c) * 1e-3;
	for (int it = 0; it < iters; it++) {
#pragma unroll
		for (int c = 0; c < kFmaChains; c++) x[c] = fma(x[c], a, b);
	}
	double t = 0;
#pragma unroll
	for (int c = 0; c < kFmaChains; c++) t += x[c];
	sink[blockIdx.x * kFmaBlock + threadIdx.x] = t;
}

}  // namespace garm

using namespace garm;

extern "C" garm_status garm_fp64_peak_selftest(int blocks_per_sm, int iters, double *tflops) {
	if (blocks_per_sm < 1 || blocks_per_sm > 16 || iters < 1 || iters > (1 << 22) || !tflops) return GARM_INVALID;
	int dev = 0, sms = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
		cudaGetLastError();
		return GARM_CUDA_ERROR;
	}
	const int blocks = sms * blocks_per_sm;
	double *sink = nullptr;
	if (cudaMalloc(&sink, size_t(blocks) * kFmaBlock * sizeof(double)) != cudaSuccess) { cudaGetLastError(); return GARM_OOM; }
	cudaStream_t st = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	garm_status r = GARM_OK;
	if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
	    cudaEventCreate(&e1) != cudaSuccess)
		r = GARM_CUDA_ERROR;
	float best = 0;
	if (r == GARM_OK) {
		// one untimed launch, then the shortest of three timed ones
		for (int rep = 0; rep < 4 && r == GARM_OK; rep++) {
			if (cudaEventRecord(e0, st) != cudaSuccess) { r = GARM_CUDA_ERROR; break; }
			kFp64Fma<<<blocks, kFmaBlock, 0, st>>>(iters, 0.999999, 1e-7, sink);
			if (cudaGetLastError() != cudaSuccess || cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
				r = GARM_CUDA_ERROR;
				break;
			}
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			if (rep > 0 && (best == 0 || ms < best)) best = ms;
		}
	}
	if (r == GARM_OK) *tflops = 2.0 * double(blocks) * kFmaBlock * kFmaChains * double(iters) / (double(best) * 1e-3) / 1e12;
	else cudaGetLastError();
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (st) cudaStreamDestroy(st);
	cudaFree(sink);
	return r;
}

extern "C" garm_status garm_barrier_selftest(int blocks, int rounds, int never_complete, double *ms_per_barrier) {
	if (blocks < 1 || rounds < 1 || rounds > (1 << 24) || (never_complete != 0 && never_complete != 1)) return GARM_INVALID;
	int dev = 0, sms = 0, perSM = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
	    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kBarrierSelftest, kSelftestBlock, 0) != cudaSuccess) {
		cudaGetLastError();
		return GARM_CUDA_ERROR;
	}
	if (blocks > sms * perSM) return GARM_INVALID;  // not co-resident
	int *mem = nullptr;  // {bar, err, passed}
	if (cudaMalloc(&mem, 16) != cudaSuccess) { cudaGetLastError(); return GARM_OOM; }
	cudaStream_t st = nullptr;
	cudaEvent_t e0 = nullptr, e1 = nullptr;
	garm_status r = GARM_OK;
	if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess || cudaEventCreate(&e0) != cudaSuccess ||
	    cudaEventCreate(&e1) != cudaSuccess || cudaMemsetAsync(mem, 0, 16, st) != cudaSuccess)
		r = GARM_CUDA_ERROR;
	int host[3] = {};
	if (r == GARM_OK) {
		unsigned *bar = reinterpret_cast<unsigned *>(mem);
		int *err = mem + 1, *passed = mem + 2;
		void *args[] = {&bar, &err, &rounds, &never_complete, &passed};
		if (cudaEventRecord(e0, st) != cudaSuccess ||
		    cudaLaunchCooperativeKernel((void *)kBarrierSelftest, dim3(blocks), dim3(kSelftestBlock), args, 0, st) != cudaSuccess ||
		    cudaEventRecord(e1, st) != cudaSuccess || cudaMemcpyAsync(host, mem, 12, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
		    cudaStreamSynchronize(st) != cudaSuccess)
			r = GARM_CUDA_ERROR;
	}
	if (r == GARM_OK) {
		float ms = 0;
		cudaEventElapsedTime(&ms, e0, e1);
		if (ms_per_barrier) *ms_per_barrier = double(ms) / (host[2] > 0 ? host[2] : 1);
		if (host[1] != 0) r = GARM_TIMEOUT;
		else if (host[2] != rounds) r = GARM_CUDA_ERROR;
	}
	if (r == GARM_CUDA_ERROR) cudaGetLastError();
	if (e0) cudaEventDestroy(e0);
	if (e1) cudaEventDestroy(e1);
	if (st) cudaStreamDestroy(st);
	cudaFree(mem);
	return r;
}
