// garm_capi.cu — the C ABI (include/garm.h): state allocation, .sav-layout
// transfers and the per-step orchestration of LevelSetLiquid<Dim>::advance
// (Source/Core/LevelSetLiquid.cpp:608-698) and ::initialize (:528-598).
#include "garm_internal.h"

#include <cmath>
#include <cstring>
#include <limits>
#include <new>

using namespace garm;

struct garm_sim {
	State s;
};

namespace {

template <typename T>
__global__ void kDeinterleave(const double *src, int ncomp, int64_t n, T *d0, T *d1, T *d2, T *d3, T *d4, T *d5, T *d6, T *d7, T *d8) {
	const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (i >= n) return;
	T *d[9] = {d0, d1, d2, d3, d4, d5, d6, d7, d8};
	for (int c = 0; c < ncomp; c++) d[c][i] = T(src[i * ncomp + c]);
}

template <typename T>
__global__ void kInterleave(double *dst, int ncomp, int64_t n, const T *d0, const T *d1, const T *d2, const T *d3, const T *d4, const T *d5, const T *d6,
                            const T *d7, const T *d8) {
	const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (i >= n) return;
	const T *d[9] = {d0, d1, d2, d3, d4, d5, d6, d7, d8};
	for (int c = 0; c < ncomp; c++) dst[i * ncomp + c] = double(d[c][i]);
}

__global__ void kSetScalar(double *p, double v) { *p = v; }
__global__ void kSetClock(double *clock, double frameLength, double cfl) { clock[0] = 0; clock[1] = frameLength; clock[2] = cfl; }
__global__ void kBeginStep(unsigned long long *counter, double *stats) {
	const unsigned long long c = ++*counter;
	double *rec = stats + ((c + kStatsCap - 1) % kStatsCap) * kStatsSlots;
	for (int q = 0; q < kStatsSlots; q++) rec[q] = 0;
}

__global__ void kPressureToCells(int64_t N, const int *grid2mat, const double *p, double *out) {
	const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (i >= N) return;
	const int r = grid2mat[i];
	out[i] = r >= 0 ? p[r] : 0.0;
}

garm_status dalloc(State &s, void **p, size_t bytes) {
	*p = nullptr;
	if (bytes == 0) return GARM_OK;
	if (s.dryRun) { s.deviceBytes += bytes; return GARM_OK; }
	if (s.nAllocs >= int(sizeof(s.allocs) / sizeof(s.allocs[0]))) return GARM_OOM;
	if (cudaMalloc(p, bytes) != cudaSuccess) { cudaGetLastError(); *p = nullptr; return GARM_OOM; }
	if (cudaMemsetAsync(*p, 0, bytes, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	s.allocs[s.nAllocs++] = *p;
	s.deviceBytes += bytes;
	return GARM_OK;
}
template <typename P>
garm_status dalloc(State &s, P **p, size_t bytes) {
	void *v = nullptr;
	const garm_status r = dalloc(s, &v, bytes);
	*p = static_cast<P *>(v);
	return r;
}

void dropGraphs(State &s);

void freeAll(State &s) {
	for (auto &g : s.stepGraph) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
	if (s.statsHost) { cudaFreeHost(s.statsHost); s.statsHost = nullptr; }
	for (int i = 0; i < s.nAllocs; i++) cudaFree(s.allocs[i]);
	s.nAllocs = 0;
	for (auto &e : s.ev) if (e) { cudaEventDestroy(e); e = nullptr; }
	for (auto &e : s.forkEv) if (e) { cudaEventDestroy(e); e = nullptr; }
	for (auto &e : s.joinEv) if (e) { cudaEventDestroy(e); e = nullptr; }
	if (s.aux) { cudaStreamDestroy(s.aux); s.aux = nullptr; }
	if (s.ownStream && s.stream) { cudaStreamDestroy(s.stream); s.stream = nullptr; }
}

garm_status allocState(State &s) {
	const size_t e = s.esz;
	const int D = s.dim;
	const size_t N = size_t(s.N);
	for (int a = 0; a < D; a++) {
		const size_t F = size_t(s.F[a]);
		GARM_TRY(dalloc(s, &s.u[a], F * e));
		GARM_TRY(dalloc(s, &s.uNew[a], F * e));
		for (int b = 0; b < D; b++) GARM_TRY(dalloc(s, &s.uGrad[a * 3 + b], F * e));
		GARM_TRY(dalloc(s, &s.fraction[a], F * e));
		GARM_TRY(dalloc(s, &s.bvel[a], F * e));
		GARM_TRY(dalloc(s, &s.normal[a], F * e));
		GARM_TRY(dalloc(s, &s.xi[a], N * e));
		GARM_TRY(dalloc(s, &s.xiNew[a], N * e));
		GARM_TRY(dalloc(s, &s.refGrad[a], N * e));
	}
	for (int q = 0; q < D * D; q++) { GARM_TRY(dalloc(s, &s.Pi[q], N * e)); GARM_TRY(dalloc(s, &s.PiNew[q], N * e)); }
	const int nm = D == 3 ? 4 : 1;
	for (int m = 0; m < nm; m++) {
		GARM_TRY(dalloc(s, &s.refMixed[m], N * e));
		for (int c = 0; c < D; c++) GARM_TRY(dalloc(s, &s.xiMixed[m * D + c], N * e));
	}
	GARM_TRY(dalloc(s, &s.phi, N * e));
	GARM_TRY(dalloc(s, &s.tmp, N * e));
	GARM_TRY(dalloc(s, &s.ori, N * e));
	GARM_TRY(dalloc(s, &s.ref, N * e));
	GARM_TRY(dalloc(s, &s.rA, N * e));
	GARM_TRY(dalloc(s, &s.rB, N * e));
	if (s.cfg.restart_newton) {
		for (int a = 0; a < D; a++) {
			GARM_TRY(dalloc(s, &s.lsGrad[a], N * e));
			GARM_TRY(dalloc(s, &s.hnGrad[a], N * e));
			GARM_TRY(dalloc(s, &s.hnPoints[a], N * e));
		}
		for (int m = 0; m < nm; m++) GARM_TRY(dalloc(s, &s.hnMixed[m], N * e));
		GARM_TRY(dalloc(s, &s.hnPhi, N * e));
		GARM_TRY(dalloc(s, (void **)&s.hnMark[0], N));
		GARM_TRY(dalloc(s, (void **)&s.hnMark[1], N));
	}
	if (s.cfg.fast_marching) {
		GARM_TRY(dalloc(s, &s.marchTent, N * e));
		GARM_TRY(dalloc(s, &s.marchTent2, N * e));
		GARM_TRY(dalloc(s, (void **)&s.marchFixed, N));
		GARM_TRY(dalloc(s, (void **)&s.marchStamp, N * 4));
		GARM_TRY(dalloc(s, (void **)&s.marchBar, 64));
		GARM_TRY(dalloc(s, (void **)&s.marchInts, 64));
	}
	GARM_TRY(dalloc(s, &s.cellDist, N * e));
	GARM_TRY(dalloc(s, &s.nodeDist, size_t(s.NN) * 8));
	GARM_TRY(dalloc(s, &s.adv, N));
	GARM_TRY(dalloc(s, &s.vis0, N));
	GARM_TRY(dalloc(s, &s.fvis0, size_t(s.Ftot)));
	GARM_TRY(dalloc(s, (void **)&s.frontBits, (size_t(s.Ftot) + 31) / 32 * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontList[0], size_t(s.Ftot) * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontList[1], size_t(s.Ftot) * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontCount, size_t(kFrontMaxPasses + 2) * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontBitsB, (size_t(s.Ftot) + 31) / 32 * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontListB[0], size_t(s.Ftot) * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontListB[1], size_t(s.Ftot) * 4));
	GARM_TRY(dalloc(s, (void **)&s.frontCountB, size_t(kFrontMaxPasses + 2) * 4));
	GARM_TRY(dalloc(s, &s.bcList, size_t(s.Ftot) * 8));
	GARM_TRY(dalloc(s, &s.bcTmp, size_t(s.Ftot) * e));
	// projection
	GARM_TRY(dalloc(s, &s.grid2mat, N * 4));
	GARM_TRY(dalloc(s, &s.mat2grid, N * 4));
	GARM_TRY(dalloc(s, &s.scanBlock, size_t(gridFor(s.N)) * 4 + 64));
	GARM_TRY(dalloc(s, &s.nUnknownsDev, 64));
	GARM_TRY(dalloc(s, &s.ent64, N * 16 * 2 * D));
	GARM_TRY(dalloc(s, &s.rowHdr, N * 4));
	GARM_TRY(dalloc(s, &s.rowIdx, N * 4 * (D == 3 ? 2 : 1)));
	GARM_TRY(dalloc(s, &s.diag, N * 8));
	GARM_TRY(dalloc(s, &s.invd, N * 8));
	GARM_TRY(dalloc(s, &s.rhs, N * 8));
	GARM_TRY(dalloc(s, &s.pres, N * 8));
	GARM_TRY(dalloc(s, &s.cgR, N * 8));
	GARM_TRY(dalloc(s, &s.cgPack[0], N * 4 * e));
	GARM_TRY(dalloc(s, &s.cgPack[1], N * 4 * e));
	if (!s.mixed) {
		GARM_TRY(dalloc(s, &s.cgP64, N * 8));
	} else {
		GARM_TRY(dalloc(s, &s.ent32, N * 8 * 2 * D));
		GARM_TRY(dalloc(s, &s.diag32, N * 4));
		GARM_TRY(dalloc(s, &s.invd32, N * 4));
		GARM_TRY(dalloc(s, &s.cgP32, N * 4));
		GARM_TRY(dalloc(s, &s.cgE32, N * 4));
	}
	s.maxBlocks = s.numSMs * 2;
	GARM_TRY(dalloc(s, &s.partials, size_t(s.maxBlocks) * 4 * 8));
	GARM_TRY(dalloc(s, &s.barrier, 64));
	GARM_TRY(dalloc(s, &s.volumeOut, 64));
	GARM_TRY(dalloc(s, &s.cgScalars, 64));
	GARM_TRY(dalloc(s, &s.cgInts, 64));
	GARM_TRY(dalloc(s, &s.redU64, 64));
	GARM_TRY(dalloc(s, &s.redI32, 64));
	GARM_TRY(dalloc(s, &s.dtDev, 64));
	GARM_TRY(dalloc(s, &s.clockDev, 64));
	GARM_TRY(dalloc(s, &s.restartFlag, 64));
	GARM_TRY(dalloc(s, &s.reinitErr, 64));
	GARM_TRY(dalloc(s, &s.stepCounter, 64));
	GARM_TRY(dalloc(s, &s.statsDev, size_t(kStatsCap) * kStatsSlots * 8));
	if (s.dryRun) return GARM_OK;
	if (cudaMallocHost(&s.statsHost, size_t(kStatsCap) * kStatsSlots * 8) != cudaSuccess) { cudaGetLastError(); s.statsHost = nullptr; return GARM_OOM; }
	// staging: the largest .sav field (Π: D*D doubles per cell)
	size_t big = N * 8 * size_t(D * D);
	if (size_t(s.Ftot) * 8 > big) big = size_t(s.Ftot) * 8;
	if (size_t(s.NN) * 8 > big) big = size_t(s.NN) * 8;
	s.stageBytes = big;
	GARM_TRY(dalloc(s, &s.stage, big));
	return GARM_OK;
}

// ---- precision/dimension dispatch ----
#define GARM_DISPATCH(S, FN, ...)                                                   \
	((S).dim == 2 ? ((S).mixed ? FN<2, float>(__VA_ARGS__) : FN<2, double>(__VA_ARGS__)) \
	              : ((S).mixed ? FN<3, float>(__VA_ARGS__) : FN<3, double>(__VA_ARGS__)))

bool validField(int f) { return f >= 0 && f < GARM_FIELD_COUNT; }

size_t fieldBytes(const State &s, int field) {
	const size_t N = size_t(s.N), D = size_t(s.dim);
	switch (field) {
	case GARM_FIELD_VELOCITY: case GARM_FIELD_FRACTION: case GARM_FIELD_BOUNDARY_VELOCITY: case GARM_FIELD_BOUNDARY_NORMAL: return size_t(s.Ftot) * 8;
	case GARM_FIELD_LEVEL_SET: case GARM_FIELD_REF_LEVEL_SET: case GARM_FIELD_ORI_LEVEL_SET: case GARM_FIELD_TMP_LEVEL_SET:
	case GARM_FIELD_CELL_DIST: case GARM_FIELD_PRESSURE: return N * 8;
	case GARM_FIELD_REF_MAP: case GARM_FIELD_REF_LEVEL_SET_GRAD: return N * 8 * D;
	case GARM_FIELD_LEVEL_SET_GRAD: return s.cfg.restart_newton ? N * 8 * D : 0;
	case GARM_FIELD_REF_MAP_GRAD: return N * 8 * D * D;
	case GARM_FIELD_ADV_REGION: return N;
	case GARM_FIELD_NODE_DIST: return size_t(s.NN) * 8;
	default: return 0;
	}
}

// Planes backing a field, in .sav component order.
int fieldPlanes(State &s, int field, void **pl, int64_t *len) {
	const int D = s.dim;
	switch (field) {
	case GARM_FIELD_VELOCITY: for (int a = 0; a < D; a++) { pl[a] = s.u[a]; len[a] = s.F[a]; } return D;
	case GARM_FIELD_FRACTION: for (int a = 0; a < D; a++) { pl[a] = s.fraction[a]; len[a] = s.F[a]; } return D;
	case GARM_FIELD_BOUNDARY_VELOCITY: for (int a = 0; a < D; a++) { pl[a] = s.bvel[a]; len[a] = s.F[a]; } return D;
	case GARM_FIELD_BOUNDARY_NORMAL: for (int a = 0; a < D; a++) { pl[a] = s.normal[a]; len[a] = s.F[a]; } return D;
	case GARM_FIELD_LEVEL_SET: pl[0] = s.phi; len[0] = s.N; return 1;
	case GARM_FIELD_REF_LEVEL_SET: pl[0] = s.ref; len[0] = s.N; return 1;
	case GARM_FIELD_ORI_LEVEL_SET: pl[0] = s.ori; len[0] = s.N; return 1;
	case GARM_FIELD_TMP_LEVEL_SET: pl[0] = s.tmp; len[0] = s.N; return 1;
	case GARM_FIELD_CELL_DIST: pl[0] = s.cellDist; len[0] = s.N; return 1;
	default: return 0;
	}
}

template <typename T>
garm_status toDevicePlanes(State &s, const double *devSrc, void **pl, int np, int64_t n) {
	T *d[9] = {};
	for (int c = 0; c < np; c++) d[c] = (T *)pl[c];
	kDeinterleave<T><<<gridFor(n), kBlock, 0, s.stream>>>(devSrc, np, n, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}
template <typename T>
garm_status fromDevicePlanes(State &s, double *devDst, void *const *pl, int np, int64_t n) {
	const T *d[9] = {};
	for (int c = 0; c < np; c++) d[c] = (const T *)pl[c];
	kInterleave<T><<<gridFor(n), kBlock, 0, s.stream>>>(devDst, np, n, d[0], d[1], d[2], d[3], d[4], d[5], d[6], d[7], d[8]); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

garm_status sync(State &s) { return cudaStreamSynchronize(s.stream) == cudaSuccess ? GARM_OK : GARM_CUDA_ERROR; }

garm_status upload(State &s, int field, const void *host, size_t bytes) {
	if (!validField(field) || !host || bytes != fieldBytes(s, field) || bytes == 0) return GARM_INVALID;
	if (field == GARM_FIELD_PRESSURE) return GARM_INVALID;
	if (field == GARM_FIELD_ADV_REGION) {
		if (cudaMemcpyAsync(s.adv, host, bytes, cudaMemcpyHostToDevice, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
		return sync(s);
	}
	if (field == GARM_FIELD_NODE_DIST) {
		if (cudaMemcpyAsync(s.nodeDist, host, bytes, cudaMemcpyHostToDevice, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
		return sync(s);
	}
	if (cudaMemcpyAsync(s.stage, host, bytes, cudaMemcpyHostToDevice, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	const double *src = (const double *)s.stage;
	void *pl[9]; int64_t len[9];
	const int np = fieldPlanes(s, field, pl, len);
	if (np > 0) {  // concatenated planes (face fields) or one cell plane
		int64_t off = 0;
		for (int c = 0; c < np; c++) {
			void *one[1] = {pl[c]};
			GARM_TRY(s.mixed ? toDevicePlanes<float>(s, src + off, one, 1, len[c]) : toDevicePlanes<double>(s, src + off, one, 1, len[c]));
			off += len[c];
		}
		return sync(s);
	}
	// interleaved per-cell vectors / matrices
	int nc = 0;
	if (field == GARM_FIELD_REF_MAP) { for (int c = 0; c < s.dim; c++) pl[c] = s.xi[c]; nc = s.dim; }
	else if (field == GARM_FIELD_REF_MAP_GRAD) { for (int c = 0; c < s.dim * s.dim; c++) pl[c] = s.Pi[c]; nc = s.dim * s.dim; }
	else if (field == GARM_FIELD_REF_LEVEL_SET_GRAD) { for (int c = 0; c < s.dim; c++) pl[c] = s.refGrad[c]; nc = s.dim; }
	else if (field == GARM_FIELD_LEVEL_SET_GRAD) { for (int c = 0; c < s.dim; c++) pl[c] = s.lsGrad[c]; nc = s.dim; }
	else return GARM_INVALID;
	GARM_TRY(s.mixed ? toDevicePlanes<float>(s, src, pl, nc, s.N) : toDevicePlanes<double>(s, src, pl, nc, s.N));
	if (field == GARM_FIELD_REF_LEVEL_SET_GRAD) GARM_TRY(GARM_DISPATCH(s, resetRefView, s));  // the view is reset after a load (LevelSetLiquid.cpp:511)
	return sync(s);
}

garm_status download(State &s, int field, void *host, size_t bytes) {
	if (!validField(field) || !host || bytes != fieldBytes(s, field) || bytes == 0) return GARM_INVALID;
	if (field == GARM_FIELD_ADV_REGION) {
		if (cudaMemcpyAsync(host, s.adv, bytes, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
		return sync(s);
	}
	if (field == GARM_FIELD_NODE_DIST) {
		if (cudaMemcpyAsync(host, s.nodeDist, bytes, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
		return sync(s);
	}
	double *dst = (double *)s.stage;
	if (field == GARM_FIELD_PRESSURE) {
		kPressureToCells<<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, s.grid2mat, s.pres, dst); s.launches++;
		GARM_CHECK_LAUNCH();
	} else {
		void *pl[9]; int64_t len[9];
		const int np = fieldPlanes(s, field, pl, len);
		if (np > 0) {
			int64_t off = 0;
			for (int c = 0; c < np; c++) {
				void *one[1] = {pl[c]};
				GARM_TRY(s.mixed ? fromDevicePlanes<float>(s, dst + off, one, 1, len[c]) : fromDevicePlanes<double>(s, dst + off, one, 1, len[c]));
				off += len[c];
			}
		} else {
			int nc = 0;
			if (field == GARM_FIELD_REF_MAP) { for (int c = 0; c < s.dim; c++) pl[c] = s.xi[c]; nc = s.dim; }
			else if (field == GARM_FIELD_REF_MAP_GRAD) { for (int c = 0; c < s.dim * s.dim; c++) pl[c] = s.Pi[c]; nc = s.dim * s.dim; }
			else if (field == GARM_FIELD_REF_LEVEL_SET_GRAD) { for (int c = 0; c < s.dim; c++) pl[c] = s.refGrad[c]; nc = s.dim; }
			else if (field == GARM_FIELD_LEVEL_SET_GRAD) { for (int c = 0; c < s.dim; c++) pl[c] = s.lsGrad[c]; nc = s.dim; }
			else return GARM_INVALID;
			GARM_TRY(s.mixed ? fromDevicePlanes<float>(s, dst, pl, nc, s.N) : fromDevicePlanes<double>(s, dst, pl, nc, s.N));
		}
	}
	if (cudaMemcpyAsync(host, dst, bytes, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	return sync(s);
}

// Outside a step the fast-marching relaxation reports its status on the host.
garm_status reinitChecked(State &s) {
	GARM_TRY(GARM_DISPATCH(s, reinitialize, s));
	return s.cfg.fast_marching ? marchStatus(s, nullptr) : tiledReinitStatus(s.stream, s.reinitErr);
}
garm_status restartChecked(State &s) {
	GARM_TRY(GARM_DISPATCH(s, restart, s));
	return s.cfg.fast_marching && s.cfg.restart_newton ? marchStatus(s, nullptr) : GARM_OK;
}

// LevelSetLiquid::initialize (LevelSetLiquid.cpp:528-598)
garm_status initialize(State &s) {
	dropGraphs(s);  // boundary work lists are baked into captured steps
	GARM_TRY(GARM_DISPATCH(s, finishBoundary, s));                       // _boundary.finish
	GARM_TRY(GARM_DISPATCH(s, enforceBoundaryLevelSet, s, s.phi, 0.0));  // enforceBoundaryLevelSet(_levelSet)
	if (s.cfg.restart_newton) GARM_TRY(GARM_DISPATCH(s, levelSetGradient, s));  // computeFirst<4>(_levelSet, _levelSetGrad)
	GARM_TRY(reinitChecked(s));                                          // reinitializeLevelSet
	GARM_TRY(GARM_DISPATCH(s, copyField, s, s.tmp, s.phi, s.N));         // _tmpLevelSet = _levelSet
	GARM_TRY(GARM_DISPATCH(s, copyField, s, s.ref, s.phi, s.N));         // _refLevelSet = _levelSet
	GARM_TRY(GARM_DISPATCH(s, copyField, s, s.ori, s.phi, s.N));         // _oriLevelSet = _levelSet
	if (s.cfg.restart_newton)                                            // _refLevelSetGrad = _levelSetGrad
		for (int a = 0; a < s.dim; a++) GARM_TRY(GARM_DISPATCH(s, copyField, s, s.refGrad[a], s.lsGrad[a], s.N));
	GARM_TRY(GARM_DISPATCH(s, resetRefView, s));                         // _refLevelSetView.reset()
	GARM_TRY(GARM_DISPATCH(s, initRefMap, s));                           // ξ = x, advRegion = 1, Π = I
	garm_step_stats st{};
	const garm_status pr = GARM_DISPATCH(s, project, s, &st);            // projectVelocity(0)
	if (pr != GARM_OK && pr != GARM_NOT_CONVERGED) return pr;
	GARM_TRY(GARM_DISPATCH(s, extrapolateToAir, s));                     // extrapolateFieldsToAir
	GARM_TRY(GARM_DISPATCH(s, enforceBoundaryConditions, s));            // _boundary.enforce(_velocity)
	s.stepIndex = 0;
	GARM_TRY(sync(s));
	return pr;
}

garm_status record(State &s, int i) { return cudaEventRecord(s.ev[i], s.stream) == cudaSuccess ? GARM_OK : GARM_CUDA_ERROR; }

// Enqueue one LevelSetLiquid::advance (LevelSetLiquid.cpp:608-698) with dt already in
// s.dtDev.  No host synchronisation: the reference-map decision is a device flag
// that gates the restart branch, and statistics go to the step's device record.
// `timed` records the stage events (not allowed inside a graph capture).
garm_status enqueueStepBody(State &s, bool timed);

garm_status enqueueStep(State &s, bool timed) {
	s.inStep = true;
	const garm_status r = enqueueStepBody(s, timed);
	s.inStep = false;
	return r;
}

garm_status enqueueStepBody(State &s, bool timed) {
	if (timed) GARM_TRY(record(s, 0));
	GARM_TRY(GARM_DISPATCH(s, advectFields, s));
	if (timed) GARM_TRY(record(s, 1));
	GARM_TRY(GARM_DISPATCH(s, generateCurrentFields, s));
	if (timed) GARM_TRY(record(s, 2));
	const bool doReinit = s.cfg.reinit_interval <= 1 || (s.stepIndex % s.cfg.reinit_interval) == 0;
	if (doReinit) GARM_TRY(GARM_DISPATCH(s, reinitialize, s));
	if (timed) GARM_TRY(record(s, 3));
	GARM_TRY(GARM_DISPATCH(s, extrapolateToCollider, s));
	if (timed) GARM_TRY(record(s, 4));
	GARM_TRY(GARM_DISPATCH(s, checkReferenceMapAsync, s, true));
	s.gate = s.restartFlag;  // restart(); generateCurrentFields(); extrapolateFieldsToCollider()  (:631-640)
	garm_status r = GARM_DISPATCH(s, restart, s);
	if (r == GARM_OK) r = GARM_DISPATCH(s, generateCurrentFields, s);
	if (r == GARM_OK) r = GARM_DISPATCH(s, extrapolateToCollider, s);
	s.gate = nullptr;
	GARM_TRY(r);
	if (timed) GARM_TRY(record(s, 5));
	GARM_TRY(GARM_DISPATCH(s, bodyForce, s));
	if (timed) GARM_TRY(record(s, 6));
	GARM_TRY(GARM_DISPATCH(s, projectAsync, s, true));
	if (timed) GARM_TRY(record(s, 7));
	GARM_TRY(GARM_DISPATCH(s, extrapolateToAir, s));
	GARM_TRY(GARM_DISPATCH(s, enforceBoundaryConditions, s));
	if (s.cfg.record_volume) GARM_TRY(GARM_DISPATCH(s, recordVolumeAsync, s));  // calculateVolume, a diagnostic
	if (timed) GARM_TRY(record(s, 8));
	s.stepIndex++;
	return GARM_OK;
}

garm_status beginStep(State &s) {
	kBeginStep<<<1, 1, 0, s.stream>>>(s.stepCounter, s.statsDev); s.launches++;
	s.hostSteps++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// dt of the step computed on the device from max|u| and the frame clock.
garm_status enqueueAutoDt(State &s) {
	GARM_TRY(GARM_DISPATCH(s, maxSpeedAsync, s));
	kStepDt<<<1, 1, 0, s.stream>>>(s.redU64, s.geom.dx, s.clockDev, s.dtDev, s.statsDev, s.stepCounter); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// Read the records of the last `k` steps into stats (the last step's record).
garm_status readRecords(State &s, int k, garm_step_stats *S) {
	if (cudaMemcpyAsync(s.statsHost, s.statsDev, size_t(kStatsCap) * kStatsSlots * 8, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	if (cudaStreamSynchronize(s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	GARM_TRY(tiledReinitStatus(s.stream, s.reinitErr));
	garm_status worst = GARM_OK;
	for (int q = 0; q < k; q++) {
		const double *rec = s.statsHost + ((s.hostSteps - 1 - q + kStatsCap) % kStatsCap) * kStatsSlots;
		if (rec[kStCgErr] != 0 || rec[kStPersistErr] == 1) return GARM_TIMEOUT;
		if (rec[kStPersistErr] != 0) return GARM_NUMERIC;
		if (rec[kStUnknowns] > 0 && !(rec[kStCgResidual] <= rec[kStCgTol])) worst = GARM_NOT_CONVERGED;
	}
	if (S) {
		const double *rec = s.statsHost + ((s.hostSteps - 1 + kStatsCap) % kStatsCap) * kStatsSlots;
		S->restarted = int(rec[kStRestarted]);
		S->rm_total = int(rec[kStRmTotal]);
		S->rm_bad = int(rec[kStRmBad]);
		S->unknowns = int(rec[kStUnknowns]);
		S->cg_iterations = int(rec[kStCgIters]);
		S->cg_refinements = int(rec[kStCgRefine]);
		S->cg_residual = rec[kStCgResidual];
		S->volume = s.cfg.record_volume ? rec[kStVolume] : 0.0;
		s.nUnknowns = S->unknowns;
	}
	return worst;
}

// LevelSetLiquid::advance (LevelSetLiquid.cpp:608-698) with a host-given dt.
garm_status advance(State &s, double dt, garm_step_stats *st) {
	garm_step_stats local{};
	garm_step_stats &S = st ? *st : local;
	std::memset(&S, 0, sizeof(S));
	GARM_TRY(beginStep(s));
	kSetScalar<<<1, 1, 0, s.stream>>>(s.dtDev, dt); s.launches++;
	GARM_CHECK_LAUNCH();
	GARM_TRY(enqueueStep(s, true));
	const garm_status pr = readRecords(s, 1, &S);
	if (pr != GARM_OK && pr != GARM_NOT_CONVERGED) return pr;
	float ms = 0;
	for (int i = 0; i < 8; i++) {
		cudaEventElapsedTime(&ms, s.ev[i], s.ev[i + 1]);
		S.ms_stage[i] = ms;
	}
	cudaEventElapsedTime(&ms, s.ev[0], s.ev[8]);
	S.ms_total = ms;
	return pr;
}

struct BufferRoles {
	void *u[3], *uNew[3], *xi[3], *xiNew[3], *Pi[9], *PiNew[9];
};
BufferRoles saveRoles(const State &s) {
	BufferRoles b;
	for (int a = 0; a < 3; a++) { b.u[a] = s.u[a]; b.uNew[a] = s.uNew[a]; b.xi[a] = s.xi[a]; b.xiNew[a] = s.xiNew[a]; }
	for (int q = 0; q < 9; q++) { b.Pi[q] = s.Pi[q]; b.PiNew[q] = s.PiNew[q]; }
	return b;
}
void restoreRoles(State &s, const BufferRoles &b) {
	for (int a = 0; a < 3; a++) { s.u[a] = b.u[a]; s.uNew[a] = b.uNew[a]; s.xi[a] = b.xi[a]; s.xiNew[a] = b.xiNew[a]; }
	for (int q = 0; q < 9; q++) { s.Pi[q] = b.Pi[q]; s.PiNew[q] = b.PiNew[q]; }
}
void swapRoles(State &s) {
	for (int a = 0; a < 3; a++) { std::swap(s.u[a], s.uNew[a]); std::swap(s.xi[a], s.xiNew[a]); }
	for (int q = 0; q < 9; q++) std::swap(s.Pi[q], s.PiNew[q]);
}

void dropGraphs(State &s) {
	for (auto &g : s.stepGraph) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
	s.graphTried = false;
	s.graphOk = false;
}

// Capture the two single-step graphs (even and odd step: the advected fields'
// ping-pong buffers alternate).  If the step cannot be captured (for example a
// cooperative launch refused in capture) the buffer roles are restored and the
// steps run as direct launches instead.
garm_status buildStepGraphs(State &s) {
	dropGraphs(s);
	s.graphTried = true;
	if (s.cfg.reinit_interval > 1) return GARM_OK;  // the captured step always reinitialises
	const BufferRoles even = saveRoles(s);
	s.evenU0 = s.u[0];
	for (int g = 0; g < 2; g++) {
		cudaGraph_t graph = nullptr;
		const long long launches = s.launches;
		const long long stepIndex = s.stepIndex;
		garm_status r = GARM_OK;
		if (cudaStreamBeginCapture(s.stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) r = GARM_CUDA_ERROR;
		else {
			kBeginStep<<<1, 1, 0, s.stream>>>(s.stepCounter, s.statsDev);
			s.launches++;
			if (cudaGetLastError() != cudaSuccess) r = GARM_CUDA_ERROR;
			if (r == GARM_OK) r = enqueueAutoDt(s);
			if (r == GARM_OK) r = enqueueStep(s, false);
			if (cudaStreamEndCapture(s.stream, &graph) != cudaSuccess) r = GARM_CUDA_ERROR;
		}
		s.graphLaunches = s.launches - launches;
		s.launches = launches;
		s.stepIndex = stepIndex;
		if (r == GARM_OK && graph && cudaGraphInstantiate(&s.stepGraph[g], graph, 0) != cudaSuccess) r = GARM_CUDA_ERROR;
		if (graph) cudaGraphDestroy(graph);
		if (r != GARM_OK) {
			cudaGetLastError();
			restoreRoles(s, even);
			dropGraphs(s);
			s.graphTried = true;
			return GARM_OK;
		}
	}
	restoreRoles(s, even);  // two captured steps swapped the roles twice
	s.graphOk = true;
	return GARM_OK;
}

// Enqueue `steps` steps with dt from the device (Simulator::advanceTimeBySteps
// policy); returns without synchronising.  ev[0]/ev[8] bracket the enqueued work.
garm_status enqueueAuto(State &s, int steps) {
	if (!s.graphTried) GARM_TRY(buildStepGraphs(s));
	GARM_TRY(record(s, 0));
	for (int k = 0; k < steps; k++) {
		if (s.graphOk) {
			// graph 0 was captured with the buffer roles of s.evenU0, graph 1 with the swapped ones
			const int parity = (s.u[0] == s.evenU0) ? 0 : 1;
			if (cudaGraphLaunch(s.stepGraph[parity], s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
			s.hostSteps++;
			s.stepIndex++;
			s.launches += s.graphLaunches;
			swapRoles(s);  // the host's view follows the graph's alternation
		} else {
			GARM_TRY(beginStep(s));
			GARM_TRY(enqueueAutoDt(s));
			GARM_TRY(enqueueStep(s, false));
		}
	}
	GARM_TRY(record(s, 8));
	s.pendingSteps = steps;
	return GARM_OK;
}

// Wait for the enqueued steps and read their records.
garm_status collect(State &s, garm_step_stats *st) {
	garm_step_stats local{};
	garm_step_stats &S = st ? *st : local;
	std::memset(&S, 0, sizeof(S));
	const int k = s.pendingSteps < 1 ? 1 : (s.pendingSteps < kStatsCap ? s.pendingSteps : kStatsCap);
	const garm_status pr = readRecords(s, k, &S);
	float ms = 0;
	cudaEventElapsedTime(&ms, s.ev[0], s.ev[8]);
	S.ms_total = ms;
	s.pendingSteps = 0;
	return pr;
}

garm_status advanceAuto(State &s, int steps, garm_step_stats *st) {
	GARM_TRY(enqueueAuto(s, steps));
	return collect(s, st);
}

}  // namespace

extern "C" {

int garm_abi_version(void) { return GARM_ABI_VERSION; }

const char *garm_status_string(garm_status st) {
	switch (st) {
	case GARM_OK: return "ok";
	case GARM_INVALID: return "invalid argument";
	case GARM_OOM: return "device out of memory";
	case GARM_NOT_CONVERGED: return "pressure solve did not converge";
	case GARM_NUMERIC: return "non-finite value";
	case GARM_CUDA_ERROR: return "CUDA error";
	case GARM_TIMEOUT: return "device-side wait timed out";
	case GARM_UNSUPPORTED: return "unsupported";
	default: return "unknown status";
	}
}

garm_status garm_config_default(garm_config *c) {
	if (!c) return GARM_INVALID;
	std::memset(c, 0, sizeof(*c));
	c->precision = GARM_PRECISION_FP64;
	c->reinit_iters = 30;
	c->reinit_cfl = 0.9;
	c->reinit_interval = 1;
	c->cg_tolerance = 1e-8;
	c->cg_max_iters = 2000;
	c->boundary_extrap_radius = 6.0;
	c->air_extrap_radius = 15.0;
	c->rm_threshold = 0.883022221559489;
	c->rm_band = 4.0;
	c->rm_ratio = 1e-5;
	c->enable_gravity = 1;
	c->mixed_residual_drop = 0.1;
	c->mixed_replace_interval = 0;
	c->cg_cells_per_block = 0;
	c->record_volume = 0;
	c->restart_newton = 0;
	c->fast_marching = 0;
	return GARM_OK;
}

// The checks a grid and a configuration pass before anything is allocated, shared by
// garm_sim_create and garm_sim_estimate_bytes (no CUDA call).
static garm_status validateRequest(const garm_grid_desc *gd, const garm_config &c) {
	if (gd->dim != 2 && gd->dim != 3) return GARM_INVALID;
	if (!(gd->spacing > 0) || gd->boundary_width < 0) return GARM_INVALID;
	for (int a = 0; a < gd->dim; a++)
		if (gd->resolution[a] < 2 * gd->boundary_width + 1 || gd->resolution[a] > (1 << 14)) return GARM_INVALID;
	// every grid (the node grid is the largest) holds fewer than 2^31 points: 32-bit indices
	int64_t nodes = 1, faces = 0;
	for (int a = 0; a < gd->dim; a++) nodes *= int64_t(gd->resolution[a]) + 1;
	for (int a = 0; a < gd->dim; a++) {
		int64_t f = 1;
		for (int b = 0; b < gd->dim; b++) f *= int64_t(gd->resolution[b]) + (b == a ? 1 : 0);
		faces += f;
	}
	if (nodes >= (int64_t(1) << 31) || faces >= (int64_t(1) << 31)) return GARM_INVALID;
	if (c.precision != GARM_PRECISION_FP64 && c.precision != GARM_PRECISION_MIXED) return GARM_INVALID;
	if (c.reinit_iters < 0 || c.cg_max_iters < 0 || !(c.cg_tolerance > 0) || c.cg_cells_per_block < 0) return GARM_INVALID;
	if (c.record_volume != 0 && c.record_volume != 1) return GARM_INVALID;
	if (c.restart_newton != 0 && c.restart_newton != 1) return GARM_INVALID;
	if (c.fast_marching != 0 && c.fast_marching != 1) return GARM_INVALID;
	// extrapolation passes are counted in a level byte
	if (!(c.boundary_extrap_radius <= 240.0) || !(c.air_extrap_radius <= 240.0)) return GARM_INVALID;
	return GARM_OK;
}

garm_status garm_sim_estimate_bytes(const garm_grid_desc *gd, const garm_config *cfg, size_t *bytes) {
	if (!gd || !bytes) return GARM_INVALID;
	garm_config c;
	if (cfg) c = *cfg; else garm_config_default(&c);
	GARM_TRY(validateRequest(gd, c));
	State s;
	s.dryRun = true;
	s.cfg = c;
	s.dim = gd->dim;
	s.mixed = c.precision == GARM_PRECISION_MIXED;
	s.esz = s.mixed ? 4 : 8;
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&s.numSMs, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) { cudaGetLastError(); s.numSMs = 160; }
	const int D = s.dim;
	int n[3];
	for (int a = 0; a < 3; a++) n[a] = a < D ? gd->resolution[a] : 1;
	s.N = int64_t(n[0]) * n[1] * n[2];
	s.NN = int64_t(n[0] + 1) * (n[1] + 1) * (D == 3 ? n[2] + 1 : 1);
	s.Ftot = 0;
	for (int a = 0; a < 3; a++) {
		s.F[a] = 0;
		if (a < D) { int64_t f = 1; for (int b = 0; b < D; b++) f *= n[b] + (b == a ? 1 : 0); s.F[a] = f; }
		s.Ftot += s.F[a];
	}
	const garm_status r = allocState(s);
	*bytes = s.deviceBytes;
	return r;
}

garm_status garm_sim_create(const garm_grid_desc *gd, const garm_config *cfg, void *stream, garm_sim **out) {
	if (!gd || !out) return GARM_INVALID;
	*out = nullptr;
	garm_config c;
	if (cfg) c = *cfg; else garm_config_default(&c);
	GARM_TRY(validateRequest(gd, c));

	garm_sim *sim = new (std::nothrow) garm_sim();
	if (!sim) return GARM_OOM;
	State &s = sim->s;
	s.cfg = c;
	s.dim = gd->dim;
	s.mixed = c.precision == GARM_PRECISION_MIXED;
	s.esz = s.mixed ? 4 : 8;
	s.geom.dim = gd->dim;
	s.geom.bw = gd->boundary_width;
	s.geom.dx = gd->spacing;
	s.geom.inv_dx = 1 / gd->spacing;
	for (int a = 0; a < 3; a++) {
		s.geom.n[a] = a < gd->dim ? gd->resolution[a] : 1;
		// StaggeredGrid origin = center - resolution * spacing / 2 (StaggeredGrid.h:32)
		s.geom.o[a] = a < gd->dim ? gd->center[a] - double(gd->resolution[a]) * gd->spacing / 2 : 0.0;
	}
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&s.numSMs, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
		cudaGetLastError();
		delete sim;
		return GARM_CUDA_ERROR;
	}
	if (stream) s.stream = (cudaStream_t)stream;
	else {
		if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess) { delete sim; return GARM_CUDA_ERROR; }
		s.ownStream = true;
	}
	for (auto &e : s.ev)
		if (cudaEventCreate(&e) != cudaSuccess) { freeAll(s); delete sim; return GARM_CUDA_ERROR; }
	if (cudaStreamCreateWithFlags(&s.aux, cudaStreamNonBlocking) != cudaSuccess) { freeAll(s); delete sim; return GARM_CUDA_ERROR; }
	for (int k = 0; k < 2; k++)
		if (cudaEventCreateWithFlags(&s.forkEv[k], cudaEventDisableTiming) != cudaSuccess ||
		    cudaEventCreateWithFlags(&s.joinEv[k], cudaEventDisableTiming) != cudaSuccess) { freeAll(s); delete sim; return GARM_CUDA_ERROR; }
	const int D = s.dim;
	s.N = int64_t(s.geom.n[0]) * s.geom.n[1] * s.geom.n[2];
	s.NN = int64_t(s.geom.n[0] + 1) * (s.geom.n[1] + 1) * (D == 3 ? s.geom.n[2] + 1 : 1);
	s.Ftot = 0;
	for (int a = 0; a < 3; a++) {
		if (a < D) {
			int64_t f = 1;
			for (int b = 0; b < D; b++) f *= s.geom.n[b] + (b == a ? 1 : 0);
			s.F[a] = f;
		} else s.F[a] = 0;
		s.Ftot += s.F[a];
	}
	garm_status r = allocState(s);
	if (r == GARM_OK) r = pcgPrepare();                                     // before any step capture
	if (r == GARM_OK && D == 3 && s.cfg.record_volume) r = loadVolumeTables();  // before any step capture
	if (r == GARM_OK) r = GARM_DISPATCH(s, initBoundary, s);           // Boundary ctor → reset()
	if (r == GARM_OK) {
		// _levelSet starts at +inf (LevelSetLiquid.cpp:49); the scene is then uploaded
		const double inf = std::numeric_limits<double>::infinity();
		double *tmpHost = nullptr;
		if (cudaMallocHost(&tmpHost, size_t(s.N) * 8) != cudaSuccess) r = GARM_OOM;
		else {
			for (int64_t i = 0; i < s.N; i++) tmpHost[i] = inf;
			r = upload(s, GARM_FIELD_LEVEL_SET, tmpHost, size_t(s.N) * 8);
			cudaFreeHost(tmpHost);
		}
	}
	if (r == GARM_OK) r = sync(s);
	if (r != GARM_OK) { freeAll(s); delete sim; return r; }
	*out = sim;
	return GARM_OK;
}

garm_status garm_sim_destroy(garm_sim *sim) {
	if (!sim) return GARM_INVALID;
	cudaStreamSynchronize(sim->s.stream);
	freeAll(sim->s);
	delete sim;
	return GARM_OK;
}

garm_status garm_sim_launch_count(const garm_sim *sim, long long *count) {
	if (!sim || !count) return GARM_INVALID;
	*count = sim->s.launches;
	return GARM_OK;
}

garm_status garm_sim_device_bytes(const garm_sim *sim, size_t *bytes) {
	if (!sim || !bytes) return GARM_INVALID;
	*bytes = sim->s.deviceBytes;
	return GARM_OK;
}

garm_status garm_sim_field_bytes(const garm_sim *sim, int field, size_t *bytes) {
	if (!sim || !bytes || !validField(field)) return GARM_INVALID;
	*bytes = fieldBytes(sim->s, field);
	return GARM_OK;
}

garm_status garm_sim_upload(garm_sim *sim, int field, const void *host, size_t bytes) { return sim ? upload(sim->s, field, host, bytes) : GARM_INVALID; }
garm_status garm_sim_download(garm_sim *sim, int field, void *host, size_t bytes) { return sim ? download(sim->s, field, host, bytes) : GARM_INVALID; }
garm_status garm_sim_initialize(garm_sim *sim) { return sim ? initialize(sim->s) : GARM_INVALID; }

garm_status garm_sim_finish_load(garm_sim *sim) {
	if (!sim) return GARM_INVALID;
	State &s = sim->s;
	dropGraphs(s);
	GARM_TRY(GARM_DISPATCH(s, finishBoundary, s));
	// ψ0 is loaded with the frame in the Newton configuration, recomputed otherwise
	// (LevelSetLiquid.cpp:500-510)
	if (s.cfg.restart_newton) GARM_TRY(GARM_DISPATCH(s, resetRefView, s));
	else GARM_TRY(GARM_DISPATCH(s, refreshRefGradient, s));
	return sync(s);
}

garm_status garm_sim_advance(garm_sim *sim, double dt, garm_step_stats *stats) {
	if (!sim || !std::isfinite(dt) || dt < 0) return GARM_INVALID;
	return advance(sim->s, dt, stats);
}

garm_status garm_sim_set_clock(garm_sim *sim, unsigned frame_rate, double cfl) {
	if (!sim || frame_rate == 0 || !(cfl > 0)) return GARM_INVALID;
	State &s = sim->s;
	kSetClock<<<1, 1, 0, s.stream>>>(s.clockDev, 1.0 / frame_rate, cfl); s.launches++;
	if (cudaGetLastError() != cudaSuccess) return GARM_CUDA_ERROR;
	return sync(s);
}

garm_status garm_sim_set_restart_override(garm_sim *sim, int mode) {
	if (!sim || mode < GARM_RESTART_AUTO || mode > GARM_RESTART_ALWAYS) return GARM_INVALID;
	State &s = sim->s;
	if (cudaMemcpyAsync(s.redI32 + kRestartOverride, &mode, sizeof(int), cudaMemcpyHostToDevice, s.stream) != cudaSuccess) {
		cudaGetLastError();
		return GARM_CUDA_ERROR;
	}
	return sync(s);
}

garm_status garm_sim_advance_auto(garm_sim *sim, int steps, garm_step_stats *stats) {
	if (!sim || steps < 1) return GARM_INVALID;
	return advanceAuto(sim->s, steps, stats);
}

garm_status garm_sim_enqueue_auto(garm_sim *sim, int steps) {
	if (!sim || steps < 1) return GARM_INVALID;
	return enqueueAuto(sim->s, steps);
}

garm_status garm_sim_poll(garm_sim *sim, int *done) {
	if (!sim || !done) return GARM_INVALID;
	const cudaError_t e = cudaEventQuery(sim->s.ev[8]);
	if (e == cudaSuccess) { *done = 1; return GARM_OK; }
	if (e == cudaErrorNotReady) { cudaGetLastError(); *done = 0; return GARM_OK; }
	return GARM_CUDA_ERROR;
}

garm_status garm_sim_collect(garm_sim *sim, garm_step_stats *stats) {
	if (!sim) return GARM_INVALID;
	return collect(sim->s, stats);
}

garm_status garm_batch_advance_auto(garm_sim *const *sims, int count, int steps, garm_step_stats *stats) {
	if (!sims || count < 1 || steps < 1) return GARM_INVALID;
	for (int i = 0; i < count; i++) if (!sims[i]) return GARM_INVALID;
	// one step of every scene per round, each on its own stream, so scenes overlap on the device
	for (int i = 0; i < count; i++) { State &s = sims[i]->s; if (!s.graphTried) GARM_TRY(buildStepGraphs(s)); GARM_TRY(record(s, 0)); }
	for (int k = 0; k < steps; k++) {
		for (int i = 0; i < count; i++) {
			State &s = sims[i]->s;
			if (s.graphOk) {
				const int parity = (s.u[0] == s.evenU0) ? 0 : 1;
				if (cudaGraphLaunch(s.stepGraph[parity], s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
				s.hostSteps++; s.stepIndex++; s.launches += s.graphLaunches;
				swapRoles(s);
			} else {
				GARM_TRY(beginStep(s));
				GARM_TRY(enqueueAutoDt(s));
				GARM_TRY(enqueueStep(s, false));
			}
		}
	}
	garm_status worst = GARM_OK;
	for (int i = 0; i < count; i++) {
		State &s = sims[i]->s;
		GARM_TRY(record(s, 8));
		s.pendingSteps = steps;
		const garm_status r = collect(s, stats ? &stats[i] : nullptr);
		if (r != GARM_OK && r != GARM_NOT_CONVERGED) return r;
		if (r == GARM_NOT_CONVERGED) worst = r;
	}
	return worst;
}

garm_status garm_sim_graph_active(const garm_sim *sim, int *active) {
	if (!sim || !active) return GARM_INVALID;
	*active = sim->s.graphOk ? 1 : 0;
	return GARM_OK;
}

garm_status garm_sim_reinit_plan(garm_sim *sim, int *form, int *threads, int *cells_per_thread, float *ms) {
	if (!sim || !form || !threads || !cells_per_thread || !ms) return GARM_INVALID;
	return GARM_DISPATCH(sim->s, reinitPlanInfo, sim->s, form, threads, cells_per_thread, ms);
}

garm_status garm_reinit_plan_set(int dim, int precision, const int *size, int form, int threads, int cells_per_thread) {
	if ((dim != 2 && dim != 3) || !size || (precision != GARM_PRECISION_FP64 && precision != GARM_PRECISION_MIXED)) return GARM_INVALID;
	for (int a = 0; a < dim; a++) if (size[a] <= 0) return GARM_INVALID;
	if (form != GARM_REINIT_CELLS && form != GARM_REINIT_COLUMNS && form != GARM_REINIT_SWEEPS && form != GARM_REINIT_TILED &&
	    form != GARM_REINIT_PAIRS && form != GARM_REINIT_PAIRS_TILED) return GARM_INVALID;
	if (threads != 0 && form != GARM_REINIT_CELLS) {
		if (cells_per_thread < 1) return GARM_INVALID;
		if (threads < 32 || threads > 256 || threads % 32 != 0) return GARM_INVALID;
	}
	return pinReinitPlan(dim, precision == GARM_PRECISION_FP64 ? 8 : 4, size, form, threads, cells_per_thread);
}

garm_status garm_sim_volume(garm_sim *sim, int evaluator_order, double *out) {
	if (!sim || !out || (evaluator_order != 0 && evaluator_order != 1)) return GARM_INVALID;
	return GARM_DISPATCH(sim->s, levelSetVolume, sim->s, evaluator_order, out);
}

garm_status garm_sim_max_speed(garm_sim *sim, double *out) {
	if (!sim || !out) return GARM_INVALID;
	return GARM_DISPATCH(sim->s, maxSpeed, sim->s, out);
}

garm_status garm_sim_time_step(garm_sim *sim, double cfl, double *dt) {
	if (!sim || !dt) return GARM_INVALID;
	double m = 0;
	GARM_TRY(garm_sim_max_speed(sim, &m));
	*dt = cfl * sim->s.geom.dx / m;  // +inf when the fluid is at rest, as the reference
	return GARM_OK;
}

#define STAGE_BODY(expr) do { if (!sim) return GARM_INVALID; State &s = sim->s; garm_status r_ = (expr); if (r_ == GARM_OK || r_ == GARM_NOT_CONVERGED) { garm_status q_ = sync(s); if (q_ != GARM_OK) return q_; } return r_; } while (0)

garm_status garm_stage_advect(garm_sim *sim, double dt) {
	if (!sim) return GARM_INVALID;
	kSetScalar<<<1, 1, 0, sim->s.stream>>>(sim->s.dtDev, dt);
	STAGE_BODY(GARM_DISPATCH(s, advectFields, s));
}
garm_status garm_stage_compose(garm_sim *sim) { STAGE_BODY(GARM_DISPATCH(s, generateCurrentFields, s)); }
garm_status garm_stage_reinit(garm_sim *sim) { STAGE_BODY(reinitChecked(s)); }
garm_status garm_stage_extrap_collider(garm_sim *sim) { STAGE_BODY(GARM_DISPATCH(s, extrapolateToCollider, s)); }
garm_status garm_stage_rm_check(garm_sim *sim, int *keep, int *total, int *bad) { STAGE_BODY(GARM_DISPATCH(s, checkReferenceMap, s, keep, total, bad)); }
garm_status garm_stage_restart(garm_sim *sim) { STAGE_BODY(restartChecked(s)); }
garm_status garm_stage_body_force(garm_sim *sim, double dt) {
	if (!sim) return GARM_INVALID;
	kSetScalar<<<1, 1, 0, sim->s.stream>>>(sim->s.dtDev, dt);
	STAGE_BODY(GARM_DISPATCH(s, bodyForce, s));
}
garm_status garm_stage_project(garm_sim *sim, garm_step_stats *stats) {
	garm_step_stats local{};
	garm_step_stats *st = stats ? stats : &local;
	std::memset(st, 0, sizeof(*st));
	STAGE_BODY(GARM_DISPATCH(s, project, s, st));
}
garm_status garm_stage_extrap_air(garm_sim *sim) { STAGE_BODY(GARM_DISPATCH(s, extrapolateToAir, s)); }
garm_status garm_stage_enforce_bc(garm_sim *sim) { STAGE_BODY(GARM_DISPATCH(s, enforceBoundaryConditions, s)); }
garm_status garm_stage_enforce_boundary_level_set(garm_sim *sim, double tol) { STAGE_BODY(GARM_DISPATCH(s, enforceBoundaryLevelSet, s, s.phi, tol)); }

garm_status garm_reinit_host(int dim, const int *size, double spacing, double *phi, int iters, double cfl, int precision) {
	if ((dim != 2 && dim != 3) || !size || !phi || !(spacing > 0) || iters < 0) return GARM_INVALID;
	if (precision != GARM_PRECISION_FP64 && precision != GARM_PRECISION_MIXED) return GARM_INVALID;
	int64_t n = 1;
	for (int a = 0; a < dim; a++) { if (size[a] <= 0 || size[a] > (1 << 14)) return GARM_INVALID; n *= size[a]; }
	if (n >= (int64_t(1) << 31)) return GARM_INVALID;  // 32-bit cell indices
	const bool f32 = precision == GARM_PRECISION_MIXED;
	const size_t e = f32 ? 4 : 8;
	// three planes, then the error flag of the tiled form on its own 16-byte line
	const size_t planes = (size_t(n) * e * 3 + 15) / 16 * 16;
	void *buf = nullptr, *stage = nullptr;
	if (cudaMalloc(&buf, planes + 16) != cudaSuccess) { cudaGetLastError(); return GARM_OOM; }
	if (cudaMalloc(&stage, size_t(n) * 8) != cudaSuccess) { cudaGetLastError(); cudaFree(buf); return GARM_OOM; }
	int *err = reinterpret_cast<int *>(static_cast<char *>(buf) + planes);
	garm_status r = GARM_OK;
	cudaStream_t st = nullptr;
	if (cudaMemset(err, 0, sizeof(int)) != cudaSuccess) r = GARM_CUDA_ERROR;
	if (r == GARM_OK && cudaMemcpy(stage, phi, size_t(n) * 8, cudaMemcpyHostToDevice) != cudaSuccess) r = GARM_CUDA_ERROR;
	if (r == GARM_OK) {
		if (f32) {
			float *p = (float *)buf;
			kDeinterleave<float><<<gridFor(n), kBlock>>>((const double *)stage, 1, n, p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
			r = dim == 2 ? reinitRaw<2, float>(st, size, spacing, p, p + n, p + 2 * n, iters, cfl, err) : reinitRaw<3, float>(st, size, spacing, p, p + n, p + 2 * n, iters, cfl, err);
			if (r == GARM_OK) kInterleave<float><<<gridFor(n), kBlock>>>((double *)stage, 1, n, p, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
		} else {
			double *p = (double *)buf;
			cudaMemcpy(p, stage, size_t(n) * 8, cudaMemcpyDeviceToDevice);
			r = dim == 2 ? reinitRaw<2, double>(st, size, spacing, p, p + n, p + 2 * n, iters, cfl, err) : reinitRaw<3, double>(st, size, spacing, p, p + n, p + 2 * n, iters, cfl, err);
			if (r == GARM_OK) cudaMemcpy(stage, p, size_t(n) * 8, cudaMemcpyDeviceToDevice);
		}
	}
	if (r == GARM_OK) r = tiledReinitStatus(st, err);
	if (r == GARM_OK && cudaMemcpy(phi, stage, size_t(n) * 8, cudaMemcpyDeviceToHost) != cudaSuccess) r = GARM_CUDA_ERROR;
	cudaFree(buf);
	cudaFree(stage);
	return r;
}

}  // extern "C"
