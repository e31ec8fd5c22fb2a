// garm_march.cu — fast-marching reinitialisation, FastMarching<Dim>::perform
// (Source/Core/FastMarching.cpp:10-128), on the GPU.
//
// The reference accepts cells one at a time from a binary heap.  Each accepted value is the
// root of the upwind quadratic over the smallest accepted neighbour per axis, and only
// values below the band width are ever accepted.  Its result is therefore the solution of
// the discrete system
//     u_i = fixed value                              on the interface (seed) cells,
//     u_i = min(band, Q(min_x u, min_y u, min_z u))  elsewhere,
// where min_a u is the smaller of the two neighbours along axis a.  Neighbours whose value
// is not below u_i drop out of Q through its own case tests, so using all neighbours gives
// the same root as using the accepted ones.  This file computes that solution without a
// heap: one persistent cooperative launch relaxes the cells, always towards smaller values
// and never below the solution, until a sweep changes nothing.  The sweeps are Jacobi
// sweeps between two buffers, so the result does not depend on the order in which blocks
// run (an in-place relaxation can settle on different last bits where a neighbour ties
// with a root), and each visits only the cells whose neighbours changed in the sweep
// before (about 140 sweeps cross a 15-cell band at 128^3, each moving a thin shell).  Each
// cell's update is the reference's quadratic in the same operation order, so the result is
// the reference's up to the last bits in exact ties, where a neighbour equal to the root
// enters or drops out of Q.
#include "garm_internal.h"
#include "garm_sync.cuh"

#include <algorithm>

namespace garm {

constexpr int kMarchBlock = 256;
constexpr int kMarchSweepCap = 4096;   // never reached on level sets; past it → GARM_NUMERIC
constexpr int kMarchCellsPerThread = 16; // blocks in proportion to the grid, so that small scenes leave SMs free


// solveQuadratic (FastMarching.cpp:112-128).  The 3-term form orders its arguments with
// the reference's two swaps, which leave p2 the largest and p0, p1 in either order.
template <typename T>
__device__ __forceinline__ T marchQuad2(T p0, T p1, T dx) {
	if (p0 > p1) { const T t = p0; p0 = p1; p1 = t; }
	if (isinf(p1) || p1 - p0 > dx) return p0 + dx;
	return ((p0 + p1) + sqrt(T(2) * dx * dx - (p0 - p1) * (p0 - p1))) * T(0.5);
}
template <typename T>
__device__ __forceinline__ T marchQuad3(T p0, T p1, T p2, T dx) {
	if (p0 > p1) { const T t = p0; p0 = p1; p1 = t; }
	if (p1 > p2) { const T t = p1; p1 = p2; p2 = t; }
	if (isinf(p2) || (p2 - p0) * (p2 - p0) + (p2 - p1) * (p2 - p1) > dx * dx) return marchQuad2(p0, p1, dx);
	const T s = p0 + p1 + p2;
	return (s + sqrt(s * s - T(3) * (p0 * p0 + p1 * p1 + p2 * p2 - dx * dx))) / T(3);
}

// std::min(a, b) as the reference uses it: b only when b < a (a NaN candidate never enters).
template <typename T>
__device__ __forceinline__ T minKeep(T a, T b) { return b < a ? b : a; }

// Seeds of perform(phi, maxSteps) (FastMarching.cpp:14-30): cells with a sign change to a
// neighbour start at the harmonic combination 1/|(1/d_x, 1/d_y, 1/d_z)| of the per-axis
// crossing distances d_a = φ/(φ - φ_nb)·dx; the others at the band width.  Both sweep
// buffers start with these values.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kMarchSeedSigns(Geom geom, const T *phi, T *tent, T *tent2, uint8_t *fixed, int *stamp, T band, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	stamp[id] = 0;
	int i, j, k;
	g.coord(id, i, j, k);
	const T f = phi[id];
	const T inf = T(INFINITY);
	T t[3] = {inf, inf, inf};
#pragma unroll
	for (int nb = 0; nb < 2 * D; nb++) {
		const int a = nb >> 1, s = (nb & 1) ? 1 : -1;
		const int ni = i + (a == 0 ? s : 0), nj = j + (a == 1 ? s : 0), nk = k + (a == 2 ? s : 0);
		if (!g.valid(ni, nj, nk)) continue;
		const T fn = phi[g.idx(ni, nj, nk)];
		if (f * fn <= T(0)) t[a] = minKeep(t[a], f / (f - fn) * g.dx);
	}
	bool any = false;
#pragma unroll
	for (int a = 0; a < D; a++) any = any || isfinite(t[a]);
	if (any) {
		T sum = T(0);
#pragma unroll
		for (int a = 0; a < D; a++) { const T r = T(1) / t[a]; sum += r * r; }
		const T v = T(1) / sqrt(sum);
		tent[id] = v;
		tent2[id] = v;
		fixed[id] = 1;
	} else {
		tent[id] = band;
		tent2[id] = band;
		fixed[id] = 0;
	}
}

// Seeds of perform(phi, maxSteps, mark) (FastMarching.cpp:46-58): marked cells keep |φ|.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kMarchSeedMarked(int64_t n, const T *phi, const uint8_t *mark, T *tent, T *tent2, uint8_t *fixed, int *stamp, T band, const int *gate) {
	if (gate && !*gate) return;
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= n) return;
	stamp[id] = 0;
	const uint8_t m = mark[id];
	const T v = m ? fabs(phi[id]) : band;
	tent[id] = v;
	tent2[id] = v;
	fixed[id] = m;
}

struct MarchCtl {
	unsigned *bar;   // grid barrier counter
	int *ints;       // [0..2] active-list sizes per sweep (rotating), [3] error (1 barrier timeout, 2 sweep cap), [4] sweeps
	int *stamp;      // per cell: the last sweep it was queued for
	int *list[2];    // active list of sweep s in list[s & 1]
	double *stats;   // step records (null outside a recorded step)
	const unsigned long long *counter;
};

// The relaxation as Jacobi sweeps over an active list.  Sweep s reads buffer s%2 and writes
// min(u, Q(neighbours)) into the other for the cells of its list; a cell that changes queues
// itself and its unseeded neighbours for sweep s+1 (once each: a per-cell stamp raised with
// atomicMax), since only their Q can change next.  Every cell outside the list of a sweep
// holds the same value in both buffers (seeds from the start; a cell that changed is in the
// next list, where it is written again), so the sweeps compute exactly the full-grid Jacobi
// iteration, and the solution is reached when a sweep changes nothing: its next list is
// empty, and both buffers then hold the solution.  The first list is the unseeded
// neighbours of seeds.  List sizes rotate over three slots: slot s%3 is read by every block
// at the start of sweep s and cleared by block 0 at the start of sweep s+1 as the size of
// sweep s+3, while sweep s+2's list is being built.
template <int D, typename T>
__global__ void __launch_bounds__(kMarchBlock) kMarch(Geom geom, T *tentA, T *tentB, const uint8_t *fixed, MarchCtl ctl, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int n = int(g.count());
	const int stride = int(gridDim.x) * blockDim.x;
	const T dx = g.dx;
	const T inf = T(INFINITY);
	unsigned epoch = 0;
	int *err = ctl.ints + 3;
	auto neighbour = [&](int id, int i, int j, int k, int q) -> int {
		const int a = q >> 1, sgn = (q & 1) ? 1 : -1;
		const int ni = i + (a == 0 ? sgn : 0), nj = j + (a == 1 ? sgn : 0), nk = k + (a == 2 ? sgn : 0);
		return g.valid(ni, nj, nk) ? int(g.idx(ni, nj, nk)) : -1;
	};
	// first list: unseeded cells next to a seed (queued for sweep 1)
	for (int base = int(blockIdx.x) * blockDim.x; base < n; base += stride) {
		const int id = base + int(threadIdx.x);
		int ids[1];
		int m = 0;
		if (id < n && !fixed[id]) {
			int i, j, k;
			g.coord(id, i, j, k);
			bool touch = false;
#pragma unroll
			for (int q = 0; q < 2 * D; q++) {
				const int nb = neighbour(id, i, j, k, q);
				if (nb >= 0 && fixed[nb]) touch = true;
			}
			if (touch) { ctl.stamp[id] = 1; ids[m++] = id; }
		}
		warpAppend(ctl.list[1], ctl.ints + 1, ids, m);
	}
	if (!gridSync(ctl.bar, err, epoch)) return;
	int sweep = 1;
	bool converged = false;
	for (; sweep <= kMarchSweepCap; sweep++) {
		const int count = *(volatile int *)(ctl.ints + sweep % 3);
		if (count == 0) { converged = true; break; }
		if (blockIdx.x == 0 && threadIdx.x == 0) ctl.ints[(sweep + 2) % 3] = 0;
		const T *src = (sweep & 1) ? tentA : tentB;
		T *dst = (sweep & 1) ? tentB : tentA;
		const int *cur = ctl.list[sweep & 1];
		int *next = ctl.list[(sweep + 1) & 1];
		int *nextCount = ctl.ints + (sweep + 1) % 3;
		for (int base = int(blockIdx.x) * blockDim.x; base < count; base += stride) {
			const int t = base + int(threadIdx.x);
			int ids[2 * D + 1];
			int m = 0;
			if (t < count) {
				const int id = cur[t];
				int i, j, k;
				g.coord(id, i, j, k);
				int nbs[2 * D];
				T mn[3] = {inf, inf, inf};
#pragma unroll
				for (int q = 0; q < 2 * D; q++) {
					nbs[q] = neighbour(id, i, j, k, q);
					if (nbs[q] >= 0) mn[q >> 1] = minKeep(mn[q >> 1], __ldcg(src + nbs[q]));
				}
				const T u = __ldcg(src + id);
				// Q exceeds its smallest argument, so with no neighbour below u the cell keeps u
				bool below = mn[0] < u || mn[1] < u;
				if (D == 3) below = below || mn[2] < u;
				T nu = u;
				if (below) {
					const T cand = D == 2 ? marchQuad2(mn[0], mn[1], dx) : marchQuad3(mn[0], mn[1], mn[2], dx);
					if (cand < u) nu = cand;
				}
				dst[id] = nu;
				if (nu < u) {
					if (atomicMax(ctl.stamp + id, sweep + 1) < sweep + 1) ids[m++] = id;
#pragma unroll
					for (int q = 0; q < 2 * D; q++)
						if (nbs[q] >= 0 && !fixed[nbs[q]] && atomicMax(ctl.stamp + nbs[q], sweep + 1) < sweep + 1) ids[m++] = nbs[q];
				}
			}
			warpAppend(next, nextCount, ids, m);
		}
		if (!gridSync(ctl.bar, err, epoch)) break;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		ctl.ints[4] = sweep;
		if (!converged && *(volatile int *)err == 0) atomicExch(err, 2);
		const int code = *(volatile int *)err;
		double *rec = stepRecord(ctl.stats, ctl.counter);
		if (rec && code) rec[kStPersistErr] = code;
	}
}

// φ = sign(φ)·tent (FastMarching.cpp:40-42, 69-71): the sign of the input, with 0 negative.
template <typename T>
__global__ void __launch_bounds__(kBlock) kMarchSign(int64_t n, T *phi, const T *tent, const int *gate) {
	if (gate && !*gate) return;
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= n) return;
	phi[id] = (phi[id] <= T(0) ? T(-1) : T(1)) * tent[id];
}

template <int D, typename T>
garm_status fastMarch(State &s, void *phiPlane, const uint8_t *mark, int maxSteps, bool record) {
	T *phi = (T *)phiPlane;
	T *tent = (T *)s.marchTent, *tent2 = (T *)s.marchTent2;
	const double bandD = maxSteps * s.geom.dx;
	// bandWidth > 0 without a mark, >= 0 with one; otherwise unbounded (FastMarching.cpp:13, 49)
	const T band = (mark ? bandD >= 0 : bandD > 0) ? T(bandD) : T(INFINITY);
	const unsigned nb = gridFor(s.N);
	if (mark) kMarchSeedMarked<D, T><<<nb, kBlock, 0, s.stream>>>(s.N, phi, mark, tent, tent2, s.marchFixed, s.marchStamp, band, s.gate);
	else kMarchSeedSigns<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, phi, tent, tent2, s.marchFixed, s.marchStamp, band, s.gate);
	s.launches++;
	GARM_CHECK_LAUNCH();
	kClearWords<<<1, 32, 0, s.stream>>>(s.marchBar, 2, (unsigned *)s.marchInts, 8); s.launches++;
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	int perSM = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kMarch<D, T>, kMarchBlock, 0);
	if (e != cudaSuccess || perSM <= 0) return GARM_CUDA_ERROR;
	// the active lists are thin shells: at most four blocks per SM, so the barrier stays cheap
	const int64_t want = (s.N + kMarchBlock * kMarchCellsPerThread - 1) / (kMarchBlock * kMarchCellsPerThread);
	const int blocks = int(std::max<int64_t>(1, std::min<int64_t>(want, std::min<int64_t>(int64_t(perSM), 4) * s.numSMs)));
	MarchCtl ctl{s.marchBar, s.marchInts, s.marchStamp, {s.frontList[0], s.frontList[1]}, record ? s.statsDev : nullptr, s.stepCounter};
	Geom geom = s.geom;
	const int *gate = s.gate;
	void *args[] = {&geom, &tent, &tent2, &s.marchFixed, &ctl, &gate};
	e = cudaLaunchCooperativeKernel((void *)kMarch<D, T>, dim3(blocks), dim3(kMarchBlock), args, 0, s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	s.launches++;
	kMarchSign<T><<<nb, kBlock, 0, s.stream>>>(s.N, phi, tent, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// Status and sweep count of the last relaxation (synchronises the stream).
garm_status marchStatus(State &s, int *sweeps) {
	int h[5] = {};
	if (cudaMemcpyAsync(h, s.marchInts, sizeof(h), cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	if (cudaStreamSynchronize(s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	if (sweeps) *sweeps = h[4];
	return h[3] == 1 ? GARM_TIMEOUT : h[3] == 2 ? GARM_NUMERIC : GARM_OK;
}

#define GARM_INST(D, T) template garm_status fastMarch<D, T>(State &, void *, const uint8_t *, int, bool);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
