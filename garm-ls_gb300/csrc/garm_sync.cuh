// garm_sync.cuh — grid-wide barrier with a bounded wait, shared by the persistent
// kernels (the pressure solve and the fast-marching relaxation).  Every kernel that
// uses it is launched cooperatively, so all of its blocks are co-resident.
#pragma once

#include <cstdint>

namespace garm {

constexpr unsigned long long kBarrierWaitNs = 2000000000ull;     // one barrier wait longer than 2 s → GARM_TIMEOUT
constexpr unsigned long long kBarrierSpinLimit = 1ull << 32;     // backstop on the number of polls

__device__ __forceinline__ unsigned ldAcquire(const unsigned *ptr) {
	unsigned v;
	asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(ptr) : "memory");
	return v;
}
__device__ __forceinline__ unsigned long long globalNs() {
	unsigned long long t;
	asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
	return t;
}
__device__ __forceinline__ void addRelease(unsigned *ptr, unsigned v) {
	asm volatile("red.release.gpu.global.add.u32 [%0], %1;" :: "l"(ptr), "r"(v) : "memory");
}

// Grid-wide barrier with a bounded wait.  Each block adds 1 to a counter with
// release semantics once its threads have passed __syncthreads; a block waits
// (acquire loads) until the counter reaches gridDim.x times the number of
// barriers passed so far.  Every poll also loads the error flag, issued first so
// that the two loads are in flight together; the flag seen with the last poll is
// handed to the block through shared memory, so leaving the barrier costs no
// further L2 round trip.  The wait is bounded in time (checked every 1024 polls
// against the global nanosecond timer): past the limit the block sets the error
// flag and returns false; every other block sees the flag while it waits at this
// barrier or the next one and returns false too.
__device__ inline bool gridSync(unsigned *bar, int *err, unsigned &epoch) {
	__shared__ int blockErr;
	__syncthreads();
	if (threadIdx.x == 0) {
		epoch += gridDim.x;
		addRelease(bar, 1u);
		unsigned long long spins = 0, start = 0;
		int e;
		for (;;) {
			e = *(volatile int *)err;
			if (ldAcquire(bar) >= epoch || e) break;
			if ((++spins & 1023ull) == 0) {
				const unsigned long long now = globalNs();
				if (start == 0) start = now;
				if (now - start > kBarrierWaitNs || spins > kBarrierSpinLimit) { atomicExch(err, 1); e = 1; break; }
			}
		}
		blockErr = e;
	}
	__syncthreads();
	return blockErr == 0;
}

// The two halves of gridSync for callers that order their block's writes themselves:
// gridArrive (thread 0 only, after a __syncthreads that follows every write of the
// phase, or after thread 0's own last write) and gridWait (every thread: thread 0 polls,
// then the block passes __syncthreads).  The reductions of the pressure solve arrive
// right after thread 0 stores the block's partial sums, which saves two block barriers
// per grid barrier.
__device__ __forceinline__ void gridArrive(unsigned *bar, unsigned &epoch) {
	epoch += gridDim.x;
	addRelease(bar, 1u);
}
__device__ inline bool gridWait(unsigned *bar, int *err, unsigned epoch) {
	__shared__ int blockErr;
	if (threadIdx.x == 0) {
		unsigned long long spins = 0, start = 0;
		int e;
		for (;;) {
			e = *(volatile int *)err;
			if (ldAcquire(bar) >= epoch || e) break;
			if ((++spins & 1023ull) == 0) {
				const unsigned long long now = globalNs();
				if (start == 0) start = now;
				if (now - start > kBarrierWaitNs || spins > kBarrierSpinLimit) { atomicExch(err, 1); e = 1; break; }
			}
		}
		blockErr = e;
	}
	__syncthreads();
	return blockErr == 0;
}

}  // namespace garm
