// garm_project.cu — Projector::project (Source/Core/Projector.cpp:13-20) on the GPU.
//   setUnknowns          (Projector.cpp:125-156)  → flag + block scan + scatter: the same
//                                                   x-fastest numbering as the serial loop
//   buildLinearSystem    (Projector.cpp:30-68)    → matrix-free rows: diag, 2D neighbour ids/weights, rhs
//   solveLinearSystem    (Projector.cpp:158-163, LinearSystem.h:23-39)
//                        → one persistent cooperative Jacobi-PCG launch (Chronopoulos–Gear form)
//                          with dot products reduced in a fixed order (deterministic): FP64 in two
//                          phases and two grid barriers per iteration; mixed as one fused FP32
//                          phase per iteration with FP64 residual replacement
//   applyPressureGradient (Projector.cpp:91-123)
#include "garm_internal.h"
#include "garm_sync.cuh"

#include <algorithm>

#include <cfloat>

namespace garm {

constexpr int kCgBlock = 512;
constexpr int kRegUnknowns = 4;  // unknowns per thread the PCG holds on chip (state in registers, rows in shared memory)

// ---------------------------------------------------------------------------
// unknown set and numbering
// ---------------------------------------------------------------------------
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kUnknownFlags(Geom geom, const T *phi, const T *fr0, const T *fr1, const T *fr2, int *flag, int *blockCount) {
	const G<D, T> cg = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	int f = 0;
	if (id < cg.count() && phi[id] <= T(0)) {
		int i, j, k; cg.coord(id, i, j, k);
		const T *fr[3] = {fr0, fr1, fr2};
#pragma unroll
		for (int q = 0; q < 2 * D; q++) {
			const int a = q >> 1, o = q & 1;
			const G<D, T> fg = faceGrid<D, T>(geom, a);
			const int64_t fid = fg.idx(i + (a == 0 ? o : 0), j + (a == 1 ? o : 0), k + (a == 2 ? o : 0));
			if (fr[a][fid] < T(1)) { f = 1; break; }
		}
	}
	if (id < cg.count()) flag[id] = f;
	const int c = __syncthreads_count(f);
	if (threadIdx.x == 0) blockCount[blockIdx.x] = c;
}

__global__ void __launch_bounds__(1024) kScanBlocks(int *counts, int nb, int *total) {
	__shared__ int sh[1024];
	const int per = (nb + blockDim.x - 1) / blockDim.x;
	const int b0 = threadIdx.x * per, b1 = min(nb, b0 + per);
	int s = 0;
	for (int b = b0; b < b1; b++) s += counts[b];
	sh[threadIdx.x] = s;
	__syncthreads();
	for (int o = 1; o < blockDim.x; o <<= 1) {  // inclusive Hillis-Steele scan
		const int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
		__syncthreads();
		sh[threadIdx.x] += v;
		__syncthreads();
	}
	int run = sh[threadIdx.x] - s;
	for (int b = b0; b < b1; b++) { const int c = counts[b]; counts[b] = run; run += c; }
	if (threadIdx.x == blockDim.x - 1) *total = sh[threadIdx.x];
}

__global__ void __launch_bounds__(kBlock) kScatterUnknowns(int64_t N, const int *blockOffset, int *grid2mat, int *mat2grid) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	const int f = (id < N) ? grid2mat[id] : 0;
	const unsigned ball = __ballot_sync(0xffffffffu, f);
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	__shared__ int wsum[kBlock / 32];
	if (lane == 0) wsum[w] = __popc(ball);
	__syncthreads();
	int off = blockOffset[blockIdx.x];
	for (int q = 0; q < w; q++) off += wsum[q];
	off += __popc(ball & ((1u << lane) - 1u));
	if (id < N) {
		if (f) { grid2mat[id] = off; mat2grid[off] = int(id); }
		else grid2mat[id] = -1;
	}
}

// One off-diagonal entry: neighbour unknown id (-1: none) and weight w (the
// matrix entry is -w), stored [k][unknown] so a warp reads one coalesced record.
struct __align__(16) NbW64 { int nb; int pad; double w; };
struct __align__(8) NbW32 { int nb; float w; };

// Compact rows, read by the solves whose unknowns outnumber what they hold on chip (those
// stream every row from memory in every iteration).  Unknowns are numbered in cell order,
// x fastest, so the neighbours of the x entries (q = 0, 1) are the unknowns i - 1 and
// i + 1, and a y neighbour lies at most one row of cells (sx) away.  The header word:
//   bits 0..2D-1   entry q present
//   bit 7          take this row's entries (neighbour and weight) from the full rows: some
//                  weight is not exactly 1, or a y distance does not fit 12 bits
//   bits 8..19     i minus the y- neighbour's id
//   bits 20..31    the y+ neighbour's id minus i
// idx holds the z neighbours' ids ([i][q - 4], 3D only).  12 bytes a row in 3D (4 in 2D)
// instead of 48 (FP32 weights) or 96 (FP64).
constexpr unsigned kRowFull = 1u << 7;
constexpr int kRowDeltaMax = 4095;
template <int NB> struct RowC { unsigned h; int2 z; };
template <int NB>
__device__ __forceinline__ RowC<NB> loadRow(const unsigned *hdr, const int *idx, int64_t i) {
	if constexpr (NB == 6) return RowC<NB>{hdr[i], reinterpret_cast<const int2 *>(idx)[i]};
	else return RowC<NB>{hdr[i], make_int2(-1, -1)};
}
// The entries of unknown i as {neighbour (-1: none), weight} (E: NbW32 or NbW64), decoded
// with selects; only a row flagged full loads its entries.
template <int NB, typename E>
__device__ __forceinline__ void decodeRow(const RowC<NB> &r, int64_t i, const E *ent, int64_t S, E (&e)[NB]) {
	const int ii = int(i);
	const int nbs[6] = {ii - 1, ii + 1, ii - int(r.h >> 8 & 0xfffu), ii + int(r.h >> 20), r.z.x, r.z.y};
#pragma unroll
	for (int k = 0; k < NB; k++) {
		e[k] = E{};
		e[k].nb = (r.h >> k & 1u) ? nbs[k] : -1;
		e[k].w = 1;
	}
	if (r.h & kRowFull) {
#pragma unroll
		for (int k = 0; k < NB; k++)
			if (r.h >> k & 1u) { const E f = ent[k * S + i]; e[k].nb = f.nb; e[k].w = f.w; }
	}
}

// ---------------------------------------------------------------------------
// rows of the ghost-fluid Poisson matrix
// ---------------------------------------------------------------------------
template <int D, typename T>
struct BuildIO {
	const T *phi;
	const T *fr[3];
	const T *u[3];
	const T *bv[3];
	const int *grid2mat;
	NbW64 *ent;
	double *diag, *invd, *rhs;
	NbW32 *ent32;
	float *diag32, *invd32;
	unsigned *hdr;
	int *idx;
	int64_t stride;
};

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kBuildSystem(Geom geom, BuildIO<D, T> io) {
	const G<D, T> cg = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= cg.count()) return;
	const int r = io.grid2mat[id];
	if (r < 0) return;
	int i, j, k; cg.coord(id, i, j, k);
	const double pc = double(io.phi[id]);
	double dg = 0, div = 0;
	unsigned hdr = 0;
	int zid[2] = {-1, -1};
#pragma unroll
	for (int q = 0; q < 2 * D; q++) {
		const int a = q >> 1, o = q & 1;
		const int side = o ? 1 : -1;
		const int ni = i + (a == 0 ? side : 0), nj = j + (a == 1 ? side : 0), nk = k + (a == 2 ? side : 0);
		const G<D, T> fg = faceGrid<D, T>(geom, a);
		const int64_t fid = fg.idx(i + (a == 0 ? o : 0), j + (a == 1 ? o : 0), k + (a == 2 ? o : 0));
		double w = 1 - double(io.fr[a][fid]);
		if (!cg.valid(ni, nj, nk)) w = 0;  // edge faces carry fraction 1 in every valid boundary
		int nb = -1; double wt = 0;
		if (w > 0) {
			const int64_t nid = cg.idx(ni, nj, nk);
			const int c = io.grid2mat[nid];
			if (c >= 0) { dg += w; nb = c; wt = w; }
			else {
				const double pn = double(io.phi[nid]);
				const double theta = pc / (pc - pn);
				dg += w * (1 / fmax(theta, .001));
			}
			div += side * w * double(io.u[a][fid]);
		}
		if (w < 1) div += side * (1 - w) * double(io.bv[a][fid]);
		io.ent[q * io.stride + r] = NbW64{nb, 0, wt};
		if (io.ent32) io.ent32[q * io.stride + r] = NbW32{nb, float(wt)};
		if (nb >= 0) {
			hdr |= 1u << q;
			if (wt != 1) hdr |= kRowFull;
			if (q == 2 || q == 3) {
				const int dist = q == 2 ? r - nb : nb - r;
				if (dist >= 1 && dist <= kRowDeltaMax) hdr |= unsigned(dist) << (q == 2 ? 8 : 20);
				else hdr |= kRowFull;
			}
		}
		if (q >= 4) zid[q - 4] = nb;
	}
	io.hdr[r] = hdr;
	if (D == 3) { io.idx[int64_t(r) * 2] = zid[0]; io.idx[int64_t(r) * 2 + 1] = zid[1]; }
	io.rhs[r] = div;
	io.diag[r] = dg;
	io.invd[r] = dg != 0 ? 1 / dg : 1;  // Eigen DiagonalPreconditioner
	if (io.diag32) { io.diag32[r] = float(dg); io.invd32[r] = dg != 0 ? float(1 / dg) : 1.0f; }
}

// ---------------------------------------------------------------------------
// persistent PCG
// ---------------------------------------------------------------------------
struct CgArgs {
	const int *nDev;
	const NbW64 *ent;
	const double *diag, *invd;
	const NbW32 *ent32;
	const float *diag32, *invd32;
	const unsigned *hdr;  // compact rows (see decodeRow)
	const int *idx;
	int64_t stride;
	const double *b;
	double *x;       // FP64 solution (pressure)
	double *r64;     // FP64 residual of the refinement loop (mixed)
	double *p64;          // FP64 form: search direction
	void *pack64[2];      // FP64 form: {r, w, s, 1/diag} per unknown, double-buffered
	float *e32, *p32;     // mixed inner solve: correction and search direction
	void *pack32[2];      // mixed inner solve: {r, w, s, 1/diag} in FP32
	double *partials;
	int maxBlocks;
	unsigned *bar;
	int *err;
	double tol;
	int maxIter;
	double drop;        // mixed: residual reduction that triggers an FP64 residual replacement
	int replaceEvery;   // mixed: replace at least every this many iterations (0: only on the drop)
	double *scal;  // [0] relative residual, [1] tolerance used
	int *ints;     // [0] matvecs, [1] refinements
};

// Vectors written by other blocks in the previous phase.  gridSync()'s acquire
// load and the block barrier after it order these plain (L1-cacheable) loads after
// the other blocks' stores; the read-only texture path (__ldg) is never used for them.
__device__ __forceinline__ double ldcg(const double *p) { return *p; }
__device__ __forceinline__ float ldcg(const float *p) { return *p; }

// Shared memory of the reductions, in doubles: [0, 48) the warp sums of a block's partials
// ([v*16 + w], as doubles or float pairs); [96, 98) reciprocals the mixed form keeps
// across iterations; [kShOut, kShOut + 8) the grid totals broadcast to the block;
// [kShStage, kShSize) the grid's partials staged for warp 0 ([v * kStageBlocks + block]).
constexpr int kShOut = 104, kShStage = 112, kStageBlocks = 256, kShSize = kShStage + 3 * kStageBlocks;

// Block partial sums of NV values → partials[v*maxBlocks + blockIdx], then the block's
// arrival at the grid barrier.  Warp sums go through shared memory to warp 0, whose lane 0
// (thread 0) stores the partials and arrives: the __syncthreads before warp 0 reads the warp
// sums orders every thread's earlier writes of the phase, and thread 0's release covers
// them.  The caller waits with gridWait.
template <int NV>
__device__ __forceinline__ void blockPartials(double (&acc)[NV], double *partials, int maxBlocks, double *sh, unsigned *bar, unsigned &epoch) {
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
	auto tree = [&](double (&t)[NV]) {
		// the NV warp sums level by level, so their shuffles and additions overlap
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			double y[NV];
#pragma unroll
			for (int v = 0; v < NV; v++) y[v] = __shfl_xor_sync(0xffffffffu, t[v], o);
#pragma unroll
			for (int v = 0; v < NV; v++) t[v] += y[v];
		}
	};
	tree(acc);
	if (lane == 0) {
#pragma unroll
		for (int v = 0; v < NV; v++) sh[v * 16 + w] = acc[v];
	}
	__syncthreads();
	if (w == 0) {
		double t[NV];
#pragma unroll
		for (int v = 0; v < NV; v++) t[v] = lane < nw ? sh[v * 16 + lane] : 0.0;
		tree(t);
		if (lane == 0) {
#pragma unroll
			for (int v = 0; v < NV; v++) partials[v * maxBlocks + blockIdx.x] = t[v];
			gridArrive(bar, epoch);
		}
	}
}

// Sum of the gridDim partials of slot v, identical in every block (a fixed partition of
// the blocks over the lanes of warp 0 and a fixed shuffle tree: deterministic).  Thread t
// loads the NV partials of block t into shared memory, so the grid's partials arrive in
// one L2 round trip; warp 0 sums them there (lane l: blocks l, l + 32, ...), lane 0 runs
// `fin` on the totals (scalar work done once per block) and the NOUT results reach the
// block through shared memory.  The next writer of the staged partials or of the results
// is this function in a later reduction, which no thread reaches before every thread has
// passed the block barriers after it.
template <int NV, int NOUT, typename Fin>
__device__ __forceinline__ void gridTotals(const double *partials, int maxBlocks, double (&out)[NOUT], double *sh, Fin fin) {
	static_assert(NOUT >= NV && NOUT <= 8 && NV <= 3, "outputs include the sums");
	const int lane = threadIdx.x & 31, nb = gridDim.x;
	double *stage = sh + kShStage;
	for (int b = threadIdx.x; b < min(nb, kStageBlocks); b += blockDim.x) {
		double q[NV];
#pragma unroll
		for (int v = 0; v < NV; v++) q[v] = ldcg(partials + v * maxBlocks + b);
#pragma unroll
		for (int v = 0; v < NV; v++) stage[v * kStageBlocks + b] = q[v];
	}
	__syncthreads();
	if (threadIdx.x < 32) {
		double t[NOUT];
#pragma unroll
		for (int v = 0; v < NV; v++) t[v] = 0;
		for (int b = lane; b < nb; b += 32) {
#pragma unroll
			for (int v = 0; v < NV; v++) t[v] += b < kStageBlocks ? stage[v * kStageBlocks + b] : ldcg(partials + v * maxBlocks + b);
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			double y[NV];
#pragma unroll
			for (int v = 0; v < NV; v++) y[v] = __shfl_xor_sync(0xffffffffu, t[v], o);
#pragma unroll
			for (int v = 0; v < NV; v++) t[v] += y[v];
		}
		if (lane == 0) {
			fin(t);
#pragma unroll
			for (int v = 0; v < NOUT; v++) sh[kShOut + v] = t[v];
		}
	}
	__syncthreads();
#pragma unroll
	for (int v = 0; v < NOUT; v++) out[v] = sh[kShOut + v];
}

struct NoFin { __device__ void operator()(double *) const {} };

// The FP64 solve's reductions, with their FP64 additions spread over one warp per SM
// sub-partition rather than a butterfly in all sixteen warps: GB300 issues a warp's FP64
// instruction about every 64 cycles per sub-partition, so the additions, not the shuffles,
// set the cost.  Block partials: every thread stages its NV values in shared memory; warps
// 0-3 each sum a quarter of them (lane l: threads l, l + 32, ... of the quarter, then the
// butterfly); lanes v < NV of warp 0 add the four quarter sums of value v in order and
// store the block's partials, and thread 0 arrives at the grid barrier (the __syncwarp
// orders lanes 1..NV-1's stores before its release).
template <int NV>
__device__ __forceinline__ void blockPartials64(double (&acc)[NV], double *partials, int maxBlocks, double *sh, unsigned *bar, unsigned &epoch) {
	static_assert(NV <= 3, "staged values");
	__shared__ double stage[3 * kCgBlock];
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, n = blockDim.x, quarter = n / 4;
#pragma unroll
	for (int v = 0; v < NV; v++) stage[v * n + threadIdx.x] = acc[v];
	__syncthreads();
	if (w < 4) {
		double t[NV];
#pragma unroll
		for (int v = 0; v < NV; v++) {
			t[v] = 0;
			for (int q = lane; q < quarter; q += 32) t[v] += stage[v * n + w * quarter + q];
		}
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			double y[NV];
#pragma unroll
			for (int v = 0; v < NV; v++) y[v] = __shfl_xor_sync(0xffffffffu, t[v], o);
#pragma unroll
			for (int v = 0; v < NV; v++) t[v] += y[v];
		}
		if (lane == 0) {
#pragma unroll
			for (int v = 0; v < NV; v++) sh[v * 16 + w] = t[v];
		}
	}
	__syncthreads();
	if (w == 0) {
		if (lane < NV) {
			double q = sh[lane * 16];
			q += sh[lane * 16 + 1];
			q += sh[lane * 16 + 2];
			q += sh[lane * 16 + 3];
			partials[lane * maxBlocks + blockIdx.x] = q;
		}
		__syncwarp();
		if (lane == 0) gridArrive(bar, epoch);
	}
}

// Grid totals for the FP64 solve: warp v sums value v's block partials (lane l: blocks l,
// l + 32, ..., then the butterfly, the order of gridTotals), so the NV sums run on
// different sub-partitions; thread 0 then runs `fin` on the totals and the NOUT results
// reach the block through shared memory.
template <int NV, int NOUT, typename Fin>
__device__ __forceinline__ void gridTotals64(const double *partials, int maxBlocks, double (&out)[NOUT], double *sh, Fin fin) {
	static_assert(NOUT >= NV && NOUT <= 8 && NV <= 3, "outputs include the sums");
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nb = gridDim.x;
	if (w < NV) {
		constexpr int U = 5;  // 160 blocks in one round trip
		double q[U];
#pragma unroll
		for (int u = 0; u < U; u++) q[u] = lane + 32 * u < nb ? ldcg(partials + w * maxBlocks + lane + 32 * u) : 0.0;
		double t = 0;
#pragma unroll
		for (int u = 0; u < U; u++)
			if (lane + 32 * u < nb) t += q[u];
		for (int b = lane + 32 * U; b < nb; b += 32) t += ldcg(partials + w * maxBlocks + b);
#pragma unroll
		for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
		if (lane == 0) sh[kShOut + w] = t;
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		double t[NOUT];
#pragma unroll
		for (int v = 0; v < NV; v++) t[v] = sh[kShOut + v];
		fin(t);
#pragma unroll
		for (int v = 0; v < NOUT; v++) sh[kShOut + v] = t[v];
	}
	__syncthreads();
#pragma unroll
	for (int v = 0; v < NOUT; v++) out[v] = sh[kShOut + v];
}

// Scalar work of an iteration is done once, by the lane that finishes the grid totals,
// and handed to the block through the broadcast totals: a decision as 0.0 / 1.0 and
// the FP32 β, α packed into the bits of one double.  The other threads read both with
// integer operations.  GB300 issues FP64 (and FP64 to FP32 conversions) at 1/64 of the
// FP32 rate, so the same scalar work in all 16 warps of a block costs microseconds per
// iteration.
__device__ __forceinline__ double packFloats(double hi, double lo) {
	return __hiloint2double(__float_as_int(float(hi)), __float_as_int(float(lo)));
}
__device__ __forceinline__ float packedHi(double p) { return __int_as_float(__double2hiint(p)); }
__device__ __forceinline__ float packedLo(double p) { return __int_as_float(__double2loint(p)); }
__device__ __forceinline__ bool flagSet(double f) { return __double_as_longlong(f) != 0; }

__device__ __forceinline__ double mulRn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float mulRn(float a, float b) { return __fmul_rn(a, b); }

// Per-unknown solver state gathered by neighbours: residual r, w = A M^-1 r,
// s = A p and the Jacobi scale 1/diag, packed so one gather touches one sector.
template <typename V> struct Pack;
template <> struct __align__(16) Pack<float> { float r, w, s, d; };
template <> struct __align__(32) Pack<double> { double r, w, s, d; };

// Both forms run preconditioned CG in the Chronopoulos–Gear arrangement (one
// global reduction per iteration), solving A e = rhs from e = 0 with the Jacobi
// preconditioner.  Mathematically it is the PCG of LinearSystem.h:23-39 (Eigen's
// algorithm, the same stopping rule |r|^2 < max(tol^2 |b|^2, DBL_MIN),
// tol = max(tol, eps/|b|)):
//     u = M^-1 r, w = A u,  γ = r·u,  δ = w·u,
//     β = γ/γ_old, α = γ / (δ - β γ / α_old),
//     p = u + β p,  s = w + β s,  x += α p,  r -= α s.
// Per-thread partial dots are reduced in a fixed order; α and β are formed in FP64
// by one lane of every block, identically in every block.

// FP64 form: the iteration in two phases.  Phase 1 updates the own unknowns (p, s,
// x, r) and publishes u = M^-1 r; after a grid barrier, phase 2 forms w = A u from
// the neighbours' published u and the three dot products, then the reduction and
// its barrier.  (The mixed form instead recomputes the neighbours' new u from their
// packed {r, w, s} to save the first barrier; in FP64 that recompute, two fma and a
// product per neighbour entry, costs more FP64-pipe time than the barrier.)
template <int NB, bool Reg>
__device__ int pcgFp64Split(const CgArgs &a, int n, double *sh, NbW64 *enS, unsigned &epoch, double *outRR, double *outB2, bool *ok) {
	using V = double;
	using E = NbW64;
	const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x, nthr = int64_t(gridDim.x) * blockDim.x;
	const int64_t S = a.stride;
	const E *__restrict__ ent = a.ent;
	const V *__restrict__ dg = a.diag;
	const V *__restrict__ invd = a.invd;
	const double *__restrict__ rhs = a.b;
	V *__restrict__ x = a.x;
	V *__restrict__ p = a.p64;
	V *__restrict__ uG = a.r64;                      // u = M^-1 r of every unknown
	Pack<V> *__restrict__ st = (Pack<V> *)a.pack64[0];  // own {r, w, s, 1/diag}; only the owner reads it
	// set-up: x = 0, r = b, s = 0, p = 0, w = A M^-1 b; partial r·u, w·u, r·r
	V acc0 = V(0), acc1 = V(0), acc2 = V(0);
	for (int64_t i = tid; i < n; i += nthr) {
		const V bi = rhs[i], di = invd[i];
		const V ui = mulRn(bi, di);
		V wi = dg[i] * ui;
#pragma unroll
		for (int k = 0; k < NB; k++) {
			const E e = ent[k * S + i];
			if (e.nb >= 0) wi = fma(-e.w, mulRn(rhs[e.nb], invd[e.nb]), wi);
		}
		x[i] = V(0); p[i] = V(0);
		st[i] = Pack<V>{bi, wi, V(0), di};
		acc0 = fma(bi, ui, acc0);
		acc1 = fma(wi, ui, acc1);
		acc2 = fma(bi, bi, acc2);
	}
	{
		double acc[3] = {acc0, acc1, acc2};
		blockPartials64<3>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
	}
	if (!gridWait(a.bar, a.err, epoch)) { *ok = false; return 0; }
	double tot[6];
	gridTotals64<3, 6>(a.partials, a.maxBlocks, tot, sh, [](double *t) { t[3] = 0; t[4] = t[0] / t[1]; t[5] = 0; });
	double gamma = tot[0];
	const double rhsNorm2 = tot[2];
	*outB2 = rhsNorm2;
	*outRR = rhsNorm2;
	if (rhsNorm2 == 0) return 0;
	const double tol = fmax(a.tol, DBL_EPSILON / sqrt(rhsNorm2));
	const double threshold = fmax(tol * tol * rhsNorm2, DBL_MIN);
	if (rhsNorm2 < threshold) return 0;

	// the register form's matrix rows, in shared memory [slot][entry][thread]
	auto en = [&](int c, int k) -> E & { return enS[(c * NB + k) * kCgBlock + threadIdx.x]; };
	V dgi[kRegUnknowns], pp[kRegUnknowns], xx[kRegUnknowns], un[kRegUnknowns];
	Pack<V> me[kRegUnknowns];
	bool own[kRegUnknowns];
	if constexpr (Reg) {
#pragma unroll
		for (int c = 0; c < kRegUnknowns; c++) {
			const int64_t i = tid + c * nthr;
			own[c] = i < n;
			pp[c] = V(0); xx[c] = V(0); un[c] = V(0);
			if (own[c]) {
				dgi[c] = dg[i];
				me[c] = st[i];
#pragma unroll
				for (int k = 0; k < NB; k++) en(c, k) = ent[k * S + i];
			} else {
				dgi[c] = V(0);
				me[c] = Pack<V>{V(0), V(0), V(0), V(0)};
#pragma unroll
				for (int k = 0; k < NB; k++) { en(c, k) = E{}; en(c, k).nb = -1; }
			}
		}
	}
	int it = 0;
	while (it < a.maxIter) {
		const double alpha = tot[4];
		const V bV = V(tot[3]), aV = V(alpha);
		// phase 1: p, s, x, r and u of the own unknowns; u published
		if constexpr (Reg) {
#pragma unroll
			for (int c = 0; c < kRegUnknowns; c++) {
				if (!own[c]) continue;
				const V ui = mulRn(me[c].r, me[c].d);
				const V pi = fma(bV, pp[c], ui);
				const V si = fma(bV, me[c].s, me[c].w);
				const V rni = fma(-aV, si, me[c].r);
				un[c] = mulRn(rni, me[c].d);
				pp[c] = pi;
				xx[c] = fma(aV, pi, xx[c]);
				me[c].r = rni; me[c].s = si;
				uG[tid + c * nthr] = un[c];
			}
		} else {
			for (int64_t i = tid; i < n; i += nthr) {
				Pack<V> m = st[i];
				const V ui = mulRn(m.r, m.d);
				const V pi = fma(bV, p[i], ui);
				const V si = fma(bV, m.s, m.w);
				const V rni = fma(-aV, si, m.r);
				uG[i] = mulRn(rni, m.d);
				p[i] = pi;
				x[i] = fma(aV, pi, x[i]);
				m.r = rni; m.s = si;
				st[i] = m;
			}
		}
		if (!gridSync(a.bar, a.err, epoch)) { *ok = false; it++; break; }
		// phase 2: w = A u from the neighbours' published u; γ = r·u, δ = w·u, |r|^2
		V g = V(0), d = V(0), rr = V(0);
		if constexpr (Reg) {
#pragma unroll
			for (int c = 0; c < kRegUnknowns; c++) {
				if (!own[c]) continue;
				V wni = dgi[c] * un[c];
#pragma unroll
				for (int k = 0; k < NB; k++)
					{ const E e = en(c, k); if (e.nb >= 0) wni = fma(-e.w, uG[e.nb], wni); }
				me[c].w = wni;
				g = fma(me[c].r, un[c], g);
				d = fma(wni, un[c], d);
				rr = fma(me[c].r, me[c].r, rr);
			}
		} else {
			// each row is loaded one unknown ahead, so that the neighbour gathers issue
			// together with the unknown's own loads
			RowC<NB> q{};
			if (tid < n) q = loadRow<NB>(a.hdr, a.idx, tid);
			for (int64_t i = tid; i < n; i += nthr) {
				const RowC<NB> row = q;
				if (i + nthr < n) q = loadRow<NB>(a.hdr, a.idx, i + nthr);
				E e[NB];
				decodeRow<NB>(row, i, ent, S, e);
				const V uni = uG[i];
				V wni = dg[i] * uni;
#pragma unroll
				for (int k = 0; k < NB; k++)
					if (e[k].nb >= 0) wni = fma(-e[k].w, uG[e[k].nb], wni);
				const V rni = st[i].r;
				st[i].w = wni;
				g = fma(rni, uni, g);
				d = fma(wni, uni, d);
				rr = fma(rni, rni, rr);
			}
		}
		double acc[3] = {g, d, rr};
		blockPartials64<3>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
		// β = γ/γ_old and α = γ/(δ - βγ/α_old) with the reciprocals of the known γ_old and
		// γ_old·α_old formed before the barrier: one division after it
		// (warp 0 alone, whose lane 0 finishes the totals)
		double invG = 0, invGA = 0;
		if (threadIdx.x < 32) { invG = 1.0 / gamma; invGA = invG / alpha; }
		if (!gridWait(a.bar, a.err, epoch)) { *ok = false; it++; break; }
		gridTotals64<3, 6>(a.partials, a.maxBlocks, tot, sh, [invG, invGA, threshold](double *t) {
			t[3] = t[0] * invG;
			t[4] = t[0] / fma(-t[0] * t[0], invGA, t[1]);
			t[5] = t[2] < threshold ? 1.0 : 0.0;  // converged
		});
		it++;
		*outRR = tot[2];
		if (flagSet(tot[5])) break;
		gamma = tot[0];
	}
	if constexpr (Reg) {
#pragma unroll
		for (int c = 0; c < kRegUnknowns; c++)
			if (own[c]) x[tid + c * nthr] = xx[c];
	}
	return it;
}

// FP64 form: one PCG on the FP64 operator.
template <int NB>
__global__ void __launch_bounds__(kCgBlock) kPcgFp64(CgArgs a) {
	__shared__ double sh[kShSize];  // reductions (see kShOut)
	const int n = *a.nDev;
	double rr = 0, b2 = 0;
	bool ok = true;
	unsigned epoch = 0;
	const int64_t nthr = int64_t(gridDim.x) * blockDim.x;
	extern __shared__ __align__(16) unsigned char pcgRows[];
	NbW64 *enS = reinterpret_cast<NbW64 *>(pcgRows);
	const int mv = n <= kRegUnknowns * nthr ? pcgFp64Split<NB, true>(a, n, sh, enS, epoch, &rr, &b2, &ok)
	                                        : pcgFp64Split<NB, false>(a, n, sh, enS, epoch, &rr, &b2, &ok);
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		a.ints[0] = mv;
		a.ints[1] = 1;
		a.scal[0] = b2 > 0 ? sqrt(rr / b2) : 0;
		a.scal[1] = b2 > 0 ? fmax(a.tol, DBL_EPSILON / sqrt(b2)) : a.tol;
	}
}

// ---------------------------------------------------------------------------
// Double-float sums on the FP32 pipe.  GB300 issues one FP64 warp instruction
// per 16 cycles per SM, so FP64-accurate dot products of FP32 vectors are
// formed instead as unevaluated pairs hi + lo of floats: each product is exact
// (a·b = p + e with e = fma(a, b, -p)) and each addition error-free (Knuth's
// TwoSum), which carries about 44 significant bits (Dekker 1971; Ogita, Rump &
// Oishi, "Accurate sum and dot product", 2005).  Only the per-block totals are
// widened to FP64.  Explicit _rn intrinsics keep the compiler from fusing the
// steps that the error terms rely on.
// ---------------------------------------------------------------------------
struct DF { float hi, lo; };
__device__ __forceinline__ DF dfTwoSum(float a, float b) {
	const float s = __fadd_rn(a, b);
	const float bb = __fsub_rn(s, a);
	return {s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ void dfAddProd(DF &acc, float a, float b) {
	const float p = __fmul_rn(a, b);
	const float e = fmaf(a, b, -p);
	const DF t = dfTwoSum(acc.hi, p);
	acc.hi = t.hi;
	acc.lo = __fadd_rn(acc.lo, __fadd_rn(t.lo, e));
}
__device__ __forceinline__ DF dfMerge(DF a, DF b) {
	const DF s = dfTwoSum(a.hi, b.hi);
	const float lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
	const float hi = __fadd_rn(s.hi, lo);
	return {hi, __fsub_rn(lo, __fsub_rn(hi, s.hi))};
}
// Scalar double-float arithmetic for the mixed solve's recurrences (β, α and the kept
// 1/γ, 1/(γα)), so that they run on the FP32 pipe: at GB300's FP64 issue rate the
// lane that forms them spent about 1 us per iteration on a chain of some 30 FP64
// instructions.  Products follow Dekker's algorithm with the exact FMA product error; the
// reciprocal is the correctly rounded FP32 reciprocal refined by one Newton–Raphson step
// on the double-float value (Joldes, Muller & Popescu, "Tight and rigorous error bounds
// for basic building blocks of double-word arithmetic", ACM TOMS 44, 2017).  Relative
// error about 2^-44, the accuracy of the double-float dot products they are formed from.
__device__ __forceinline__ DF dfQuick(float hi, float lo) {  // renormalise (|hi| >= |lo|)
	const float s = __fadd_rn(hi, lo);
	return {s, __fsub_rn(lo, __fsub_rn(s, hi))};
}
__device__ __forceinline__ DF dfMul(DF a, DF b) {
	const float p = __fmul_rn(a.hi, b.hi);
	float e = fmaf(a.hi, b.hi, -p);
	e = fmaf(a.hi, b.lo, e);
	e = fmaf(a.lo, b.hi, e);
	return dfQuick(p, e);
}
__device__ __forceinline__ DF dfNeg(DF a) { return {-a.hi, -a.lo}; }
__device__ __forceinline__ DF dfRecip(DF b) {
	const float y = __frcp_rn(b.hi);
	const float r = fmaf(-b.lo, y, fmaf(-b.hi, y, 1.0f));  // 1 - b·y
	return dfQuick(y, __fmul_rn(y, r));
}
// a < b for normalised double-floats
__device__ __forceinline__ bool dfLess(DF a, DF b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ DF dfFromDouble(double x) { const float hi = float(x); return {hi, float(x - double(hi))}; }
__device__ __forceinline__ double dfToDouble(DF a) { return double(a.hi) + double(a.lo); }
// A double-float carried in the bits of one double: broadcast through shared memory and
// kept across iterations without FP64 instructions.
__device__ __forceinline__ double dfPack(DF a) { return __hiloint2double(__float_as_int(a.hi), __float_as_int(a.lo)); }
__device__ __forceinline__ DF dfUnpack(double p) { return {__int_as_float(__double2hiint(p)), __int_as_float(__double2loint(p))}; }

__device__ __forceinline__ DF dfWarpSum(DF v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v = dfMerge(v, DF{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)});
	return v;
}
// NV warp sums level by level, so the shuffles and merges of the values overlap.
template <int NV>
__device__ __forceinline__ void dfWarpSumN(DF (&v)[NV]) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		DF w[NV];
#pragma unroll
		for (int q = 0; q < NV; q++) w[q] = DF{__shfl_xor_sync(0xffffffffu, v[q].hi, o), __shfl_xor_sync(0xffffffffu, v[q].lo, o)};
#pragma unroll
		for (int q = 0; q < NV; q++) v[q] = dfMerge(v[q], w[q]);
	}
}
// Block sums of NV double-float values → partials (as float pairs) [v*maxBlocks + blockIdx],
// then the block's arrival at the grid barrier, as blockPartials.
template <int NV>
__device__ __forceinline__ void blockPartialsDF(DF (&acc)[NV], double *partials, int maxBlocks, double *sh, unsigned *bar, unsigned &epoch) {
	float2 *s2 = reinterpret_cast<float2 *>(sh);
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
	dfWarpSumN<NV>(acc);
	if (lane == 0) {
#pragma unroll
		for (int v = 0; v < NV; v++) s2[v * 16 + w] = make_float2(acc[v].hi, acc[v].lo);
	}
	__syncthreads();
	if (w == 0) {
		float2 *p2 = reinterpret_cast<float2 *>(partials);
		DF x[NV];
#pragma unroll
		for (int v = 0; v < NV; v++) {
			x[v] = DF{0.f, 0.f};
			if (lane < nw) { const float2 q = s2[v * 16 + lane]; x[v] = DF{q.x, q.y}; }
		}
		dfWarpSumN<NV>(x);
		if (lane == 0) {
#pragma unroll
			for (int v = 0; v < NV; v++) p2[v * maxBlocks + blockIdx.x] = make_float2(x[v].hi, x[v].lo);
			gridArrive(bar, epoch);
		}
	}
}
// Grid totals of NV double-float partials for the mixed solve's iterations, without the
// widening to FP64: warp 0 loads every block's partials itself, lane l those of blocks
// l, l + 32, ... all at once (one L2 round trip, no staging), and sums them in that fixed
// order and a fixed shuffle tree; lane 0 hands the NV totals to
// fin(const DF *totals, double *out), which fills the NOUT words broadcast to the block
// through shared memory.
template <int NV, int NOUT, typename Fin>
__device__ __forceinline__ void gridTotalsDFRaw(const double *partials, int maxBlocks, double (&out)[NOUT], double *sh, Fin fin) {
	static_assert(NOUT <= 8 && NV <= 3, "broadcast words");
	const int lane = threadIdx.x & 31, nb = gridDim.x;
	const float2 *p2 = reinterpret_cast<const float2 *>(partials);  // ordered by the grid barrier, as ldcg
	if (threadIdx.x < 32) {
		DF x[NV];
#pragma unroll
		for (int v = 0; v < NV; v++) x[v] = DF{0.f, 0.f};
		constexpr int U = 5;  // 160 blocks in one round trip
		float2 q[U][NV];
#pragma unroll
		for (int u = 0; u < U; u++)
#pragma unroll
			for (int v = 0; v < NV; v++) q[u][v] = lane + 32 * u < nb ? p2[v * maxBlocks + lane + 32 * u] : make_float2(0.f, 0.f);
#pragma unroll
		for (int u = 0; u < U; u++)
#pragma unroll
			for (int v = 0; v < NV; v++) x[v] = dfMerge(x[v], DF{q[u][v].x, q[u][v].y});
		for (int b = lane + 32 * U; b < nb; b += 32) {
#pragma unroll
			for (int v = 0; v < NV; v++) { const float2 r = p2[v * maxBlocks + b]; x[v] = dfMerge(x[v], DF{r.x, r.y}); }
		}
		dfWarpSumN<NV>(x);
		if (lane == 0) {
			double t[NOUT];
			fin(x, t);
#pragma unroll
			for (int v = 0; v < NOUT; v++) sh[kShOut + v] = t[v];
		}
	}
	__syncthreads();
#pragma unroll
	for (int v = 0; v < NOUT; v++) out[v] = sh[kShOut + v];
}

// Power of two s with s·rms(r) in [1, 2): the FP32 system is solved for s·r so
// its values, products and sums stay far from the FP32 range limits whatever
// the scale of the pressure equation.
__device__ __forceinline__ double unitScale(double sumSq, int n) {
	const double rms = sqrt(sumSq / double(n > 0 ? n : 1));
	return rms > 0 ? ldexp(1.0, -ilogb(rms)) : 1.0;
}

// Mixed form: one FP32 PCG (the Chronopoulos–Gear iteration above in one fused
// phase per iteration: each thread updates its own unknowns and recomputes, from
// last iteration's packed {r, w, s} of its neighbours, their new u with the owner's
// fma/mul sequence, so bit-identically, which gives w = A u without a second
// barrier; the packed state is double-buffered.  FP32 vectors and element arithmetic,
// double-float dot products and scalar recurrences) with FP64 residual replacement (van der Vorst & Ye,
// "Residual replacement strategies for Krylov subspace iterative methods",
// SIAM J. Sci. Comput. 22, 2000, as used by reliable-update mixed-precision CG).
// The FP32 iterates x32 are a scaled correction to the FP64 solution x64.
// Whenever the recursive residual has dropped by the factor `drop` since the
// last replacement, or looks converged:
//   x64 += x32/s, x32 = 0;  r = b - A64 x64 in FP64 (the convergence test uses
//   this true residual only);  new scale s';  r32 = s' r;  u = M^-1 r32 and
//   w = A32 u recomputed;  p, s·A p and γ_old rescaled by s'/s (exact);
// and the iteration continues with the same search direction, β and α formed
// from the new γ = r·u, δ = w·u by the usual recurrences.  No Krylov
// information is discarded, so the iteration count stays close to the FP64
// solver's, while the residual the solve reports is FP64-exact.
template <int NB, bool Reg>
__device__ void pcgMixedReplace(const CgArgs &a, int n, double *sh, NbW32 *enS, unsigned &epoch, int &itOut, int &replOut, double &relOut, double &tolOut) {
	using V = float;
	using E = NbW32;
	const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x, nthr = int64_t(gridDim.x) * blockDim.x;
	const int64_t S = a.stride;
	const E *__restrict__ ent = a.ent32;
	const V *__restrict__ invd = a.invd32;
	const V *__restrict__ dg = a.diag32;
	Pack<V> *stb[2] = {(Pack<V> *)a.pack32[0], (Pack<V> *)a.pack32[1]};
	V *__restrict__ x32 = a.e32;
	V *__restrict__ p32 = a.p32;
	itOut = 0; replOut = 0; relOut = 0; tolOut = a.tol;
	// |b|^2 in FP64 (sets the tolerance and the first scale)
	{
		double acc[1] = {0};
		for (int64_t i = tid; i < n; i += nthr) { const double b = a.b[i]; acc[0] += b * b; }
		blockPartials<1>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
	}
	if (!gridWait(a.bar, a.err, epoch)) return;
	double b2v[1];
	gridTotals<1, 1>(a.partials, a.maxBlocks, b2v, sh, NoFin{});
	const double b2 = b2v[0];
	if (b2 == 0) return;
	const double tol = fmax(a.tol, DBL_EPSILON / sqrt(b2));
	const double threshold = fmax(tol * tol * b2, DBL_MIN);
	tolOut = tol;
	relOut = 1;
	if (b2 < threshold) { relOut = 0; return; }
	double scale = unitScale(b2, n);
	// set-up: x64 = x32 = p = s = 0, r = scale·b, u = M^-1 r, w = A u
	{
		DF acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
		for (int64_t i = tid; i < n; i += nthr) {
			const V bi = V(a.b[i] * scale), di = invd[i];
			const V ui = mulRn(bi, di);
			V wi = dg[i] * ui;
#pragma unroll
			for (int k = 0; k < NB; k++) {
				const E e = ent[k * S + i];
				if (e.nb >= 0) wi = fma(-e.w, mulRn(V(a.b[e.nb] * scale), invd[e.nb]), wi);
			}
			a.x[i] = 0; x32[i] = V(0); p32[i] = V(0);
			stb[0][i] = Pack<V>{bi, wi, V(0), di};
			dfAddProd(acc[0], bi, ui);
			dfAddProd(acc[1], wi, ui);
		}
		blockPartialsDF<2>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
	}
	if (!gridWait(a.bar, a.err, epoch)) return;
	// tot, broadcast as bits: γ and α as double-floats, the replacement decision (non-zero:
	// replace), the FP32 β and α packed.  The lane that finishes the totals also keeps 1/γ
	// and 1/(γα), as double-floats, for the next iteration's β and α in sh[96], sh[97],
	// which no reduction touches.
	double tot[4];
	gridTotalsDFRaw<2, 4>(a.partials, a.maxBlocks, tot, sh, [sh](const DF *x, double *t) {
		const DF ig = dfRecip(x[0]), al = dfMul(x[0], dfRecip(x[1]));
		t[0] = dfPack(x[0]); t[1] = dfPack(al); t[2] = 0; t[3] = dfPack(DF{0.f, al.hi});
		sh[96] = dfPack(ig); sh[97] = dfPack(dfMul(ig, dfRecip(al)));
	});
	const double drop2 = a.drop * a.drop;
	const int maxIter = a.maxIter, replaceEvery = a.replaceEvery;
	double gamma = tot[0], lastTrue = b2;  // gamma: γ as a packed double-float
	// replaced once |r|^2 of the scaled system falls below max(drop^2 |r_true|^2, threshold)·s^2
	DF limit = dfFromDouble(fmax(drop2 * lastTrue, threshold) * (scale * scale));
	int cur = 0, it = 0, lastReplace = 0;
	// on-chip copies (used when every thread owns at most kRegUnknowns unknowns)
	// the register form's matrix rows, in shared memory [slot][entry][thread]
	auto en = [&](int c, int k) -> E & { return enS[(c * NB + k) * kCgBlock + threadIdx.x]; };
	V dgi[kRegUnknowns], pp[kRegUnknowns], xx[kRegUnknowns];
	Pack<V> me[kRegUnknowns];
	bool own[kRegUnknowns];
	if constexpr (Reg) {
#pragma unroll
		for (int c = 0; c < kRegUnknowns; c++) {
			const int64_t i = tid + c * nthr;
			own[c] = i < n;
			pp[c] = V(0); xx[c] = V(0);
			if (own[c]) {
				me[c] = stb[0][i];
				dgi[c] = dg[i];
#pragma unroll
				for (int k = 0; k < NB; k++) en(c, k) = ent[k * S + i];
			} else {
				dgi[c] = V(0);
				me[c] = Pack<V>{V(0), V(0), V(0), V(0)};
#pragma unroll
				for (int k = 0; k < NB; k++) { en(c, k) = E{}; en(c, k).nb = -1; }
			}
		}
	}
	while (it < a.maxIter) {
		// ---- one fused C-G iteration ----
		const double alphaPacked = tot[1];
		const V bV = packedHi(tot[3]), aV = packedLo(tot[3]);
		{
			const Pack<V> *__restrict__ sc = stb[cur];
			Pack<V> *__restrict__ sn = stb[cur ^ 1];
			DF acc[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
			auto update = [&](const Pack<V> &m, V dgI, V pOld, V xOld, auto entry, Pack<V> &mOut, V &pOut, V &xOut) {
				const V ui = mulRn(m.r, m.d);
				const V pi = fma(bV, pOld, ui);
				const V si = fma(bV, m.s, m.w);
				const V rni = fma(-aV, si, m.r);
				const V uni = mulRn(rni, m.d);
				V wni = dgI * uni;
#pragma unroll
				for (int k = 0; k < NB; k++) {
					const E e = entry(k);
					if (e.nb >= 0) {
						const Pack<V> q = sc[e.nb];
						const V snb = fma(bV, q.s, q.w);
						const V rnb = fma(-aV, snb, q.r);
						wni = fma(-e.w, mulRn(rnb, q.d), wni);
					}
				}
				pOut = pi;
				xOut = fma(aV, pi, xOld);
				mOut = Pack<V>{rni, wni, si, m.d};
				dfAddProd(acc[0], rni, uni);
				dfAddProd(acc[1], wni, uni);
				dfAddProd(acc[2], rni, rni);
			};
			if constexpr (Reg) {
#pragma unroll
				for (int c = 0; c < kRegUnknowns; c++) {
					if (!own[c]) continue;
					update(me[c], dgi[c], pp[c], xx[c], [&](int k) { return en(c, k); }, me[c], pp[c], xx[c]);
					sn[tid + c * nthr] = me[c];
				}
			} else {
				int64_t i = tid;
				for (; i + nthr < n; i += 2 * nthr) {
					const int64_t j = i + nthr;
					Pack<V> m0 = sc[i], m1 = sc[j];
					V p0 = p32[i], x0 = x32[i], p1 = p32[j], x1 = x32[j];
					const V d0 = dg[i], d1 = dg[j];
					E e0[NB], e1[NB];
					decodeRow<NB>(loadRow<NB>(a.hdr, a.idx, i), i, ent, S, e0);
					decodeRow<NB>(loadRow<NB>(a.hdr, a.idx, j), j, ent, S, e1);
					update(m0, d0, p0, x0, [&](int k) { return e0[k]; }, m0, p0, x0);
					update(m1, d1, p1, x1, [&](int k) { return e1[k]; }, m1, p1, x1);
					sn[i] = m0; p32[i] = p0; x32[i] = x0;
					sn[j] = m1; p32[j] = p1; x32[j] = x1;
				}
				if (i < n) {
					E e0[NB];
					decodeRow<NB>(loadRow<NB>(a.hdr, a.idx, i), i, ent, S, e0);
					Pack<V> m = sc[i];
					V pv = p32[i], xv = x32[i];
					update(m, dg[i], pv, xv, [&](int k) { return e0[k]; }, m, pv, xv);
					sn[i] = m; p32[i] = pv; x32[i] = xv;
				}
			}
			cur ^= 1;
			blockPartialsDF<3>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
		}
		// β = γ/γ_old and α = γ/den, den = δ - βγ/α_old = δ - γ²/(γ_old α_old), from the
		// kept 1/γ_old and 1/(γ_old α_old).  One reciprocal, of q = γ·den, gives α = γ²/q
		// and the next pair: 1/γ = den/q and 1/(γα) = den/γ², all in double-float
		// arithmetic.  The same lane decides whether the residual is replaced after this
		// iteration.
		const double gOldPacked = gamma;
		if (!gridWait(a.bar, a.err, epoch)) break;
		const int itNext = it + 1;
		gridTotalsDFRaw<3, 4>(a.partials, a.maxBlocks, tot, sh, [=](const DF *x, double *t) {
			const DF g = x[0];
			const DF beta = dfMul(g, dfUnpack(sh[96]));
			const DF gg = dfMul(g, g);
			const DF den = dfMerge(x[1], dfNeg(dfMul(gg, dfUnpack(sh[97]))));
			const DF rq = dfRecip(dfMul(g, den));
			const DF al = dfMul(gg, rq);
			const DF invG = dfMul(den, rq);
			sh[96] = dfPack(invG);
			sh[97] = dfPack(dfMul(dfMul(invG, invG), den));
			const bool due = replaceEvery > 0 && itNext - lastReplace >= replaceEvery;
			t[0] = dfPack(g);
			t[1] = dfPack(al);
			t[2] = (dfLess(x[2], limit) || itNext >= maxIter || due) ? 1.0 : 0.0;
			t[3] = dfPack(DF{beta.hi, al.hi});  // packedHi: β, packedLo: α
		});
		it = itNext;
		gamma = tot[0];
		if (!flagSet(tot[2])) continue;
		lastReplace = it;

		// ---- residual replacement ----
		// (1) fold the scaled FP32 correction into the FP64 solution
		const double inv = 1.0 / scale;  // a power of two: exact
		if constexpr (Reg) {
#pragma unroll
			for (int c = 0; c < kRegUnknowns; c++)
				if (own[c]) { const int64_t i = tid + c * nthr; a.x[i] += double(xx[c]) * inv; xx[c] = V(0); }
		} else {
			for (int64_t i = tid; i < n; i += nthr) { a.x[i] += double(x32[i]) * inv; x32[i] = V(0); }
		}
		if (!gridSync(a.bar, a.err, epoch)) break;
		// (2) r = b - A64 x64 in FP64
		{
			double acc2[1] = {0};
			for (int64_t i = tid; i < n; i += nthr) {
				double ax = a.diag[i] * a.x[i];
#pragma unroll
				for (int k = 0; k < NB; k++) {
					const NbW64 e = a.ent[k * S + i];
					if (e.nb >= 0) ax -= e.w * a.x[e.nb];
				}
				const double ri = a.b[i] - ax;
				a.r64[i] = ri;
				acc2[0] += ri * ri;
			}
			blockPartials<1>(acc2, a.partials, a.maxBlocks, sh, a.bar, epoch);
		}
		if (!gridWait(a.bar, a.err, epoch)) break;
		double tr[1];
		gridTotals<1, 1>(a.partials, a.maxBlocks, tr, sh, NoFin{});
		replOut++;
		relOut = sqrt(tr[0] / b2);
		if (tr[0] < threshold || it >= a.maxIter) break;
		lastTrue = tr[0];
		// (3) rescale; r32 = s' r; u = M^-1 r32, w = A32 u; p and s·A p follow the scale
		const double newScale = unitScale(tr[0], n);
		const V ratio = V(newScale / scale);  // a power of two
		const double ratio2 = (newScale / scale) * (newScale / scale);
		scale = newScale;
		limit = dfFromDouble(fmax(drop2 * lastTrue, threshold) * (scale * scale));
		{
			const Pack<V> *__restrict__ sc = stb[cur];
			Pack<V> *__restrict__ sn = stb[cur ^ 1];
			DF acc[2] = {{0.f, 0.f}, {0.f, 0.f}};
			auto rebuild = [&](int64_t i, const Pack<V> &m, V dgI, auto entry) {
				const V ri = V(a.r64[i] * scale);
				const V ui = mulRn(ri, m.d);
				V wi = dgI * ui;
#pragma unroll
				for (int k = 0; k < NB; k++) {
					const E e = entry(k);
					if (e.nb >= 0) wi = fma(-e.w, mulRn(V(a.r64[e.nb] * scale), sc[e.nb].d), wi);
				}
				dfAddProd(acc[0], ri, ui);
				dfAddProd(acc[1], wi, ui);
				return Pack<V>{ri, wi, m.s * ratio, m.d};
			};
			if constexpr (Reg) {
#pragma unroll
				for (int c = 0; c < kRegUnknowns; c++)
					if (own[c]) {
						const int64_t i = tid + c * nthr;
						me[c] = rebuild(i, me[c], dgi[c], [&](int k) { return en(c, k); });
						pp[c] *= ratio;
						sn[i] = me[c];
					}
			} else {
				for (int64_t i = tid; i < n; i += nthr) {
					const Pack<V> m = sc[i];
					sn[i] = rebuild(i, m, dg[i], [&](int k) { return ent[k * S + i]; });
					p32[i] *= ratio;
				}
			}
			cur ^= 1;
			blockPartialsDF<2>(acc, a.partials, a.maxBlocks, sh, a.bar, epoch);
		}
		if (!gridWait(a.bar, a.err, epoch)) break;
		gridTotalsDFRaw<2, 4>(a.partials, a.maxBlocks, tot, sh, [gOldPacked, ratio2, alphaPacked, sh](const DF *x, double *t) {
			// β and α after a replacement in FP64 (a few times per solve)
			const double g = dfToDouble(x[0]), d = dfToDouble(x[1]);
			const double beta = g / (dfToDouble(dfUnpack(gOldPacked)) * ratio2);
			const double al = g / (d - beta * g / dfToDouble(dfUnpack(alphaPacked)));
			t[0] = dfPack(x[0]);
			t[1] = dfPack(dfFromDouble(al));
			t[2] = 0;
			t[3] = packFloats(beta, al);
			sh[96] = dfPack(dfFromDouble(1.0 / g));
			sh[97] = dfPack(dfFromDouble(1.0 / (g * al)));
		});
		gamma = tot[0];
	}
	itOut = it;
}
template <int NB>
__global__ void __launch_bounds__(kCgBlock) kPcgMixed(CgArgs a) {
	__shared__ double sh[kShSize];  // reductions (see kShOut)
	const int n = *a.nDev;
	unsigned epoch = 0;
	int it = 0, repl = 0;
	double rel = 0, tolUsed = a.tol;
	const int64_t nthr = int64_t(gridDim.x) * blockDim.x;
	extern __shared__ __align__(16) unsigned char pcgRows[];
	NbW32 *enS = reinterpret_cast<NbW32 *>(pcgRows);
	if (n <= kRegUnknowns * nthr) pcgMixedReplace<NB, true>(a, n, sh, enS, epoch, it, repl, rel, tolUsed);
	else pcgMixedReplace<NB, false>(a, n, sh, enS, epoch, it, repl, rel, tolUsed);
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		a.ints[0] = it;
		a.ints[1] = repl;
		a.scal[0] = rel;
		a.scal[1] = tolUsed;
	}
}

// ---------------------------------------------------------------------------
// pressure gradient
// ---------------------------------------------------------------------------
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kApplyPressure(Geom geom, T *u0, T *u1, T *u2, const T *phi, const int *grid2mat, const double *p, int64_t F0, int64_t F1, int64_t Ftot) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, T> fg = faceGrid<D, T>(geom, axis);
	const G<D, T> cg = cellGrid<D, T>(geom);
	int i, j, k; fg.coord(id, i, j, k);
	const int i0 = i - (axis == 0), j0 = j - (axis == 1), k0 = k - (axis == 2);
	if (!cg.valid(i0, j0, k0) || !cg.valid(i, j, k)) return;
	const int64_t c0 = cg.idx(i0, j0, k0), c1 = cg.idx(i, j, k);
	const int id0 = grid2mat[c0], id1 = grid2mat[c1];
	if (id0 < 0 && id1 < 0) return;
	const double p0 = id0 >= 0 ? p[id0] : 0;
	const double p1 = id1 >= 0 ? p[id1] : 0;
	T *u = axis == 0 ? u0 : (axis == 1 ? u1 : u2);
	if (id0 >= 0 && id1 >= 0) { u[id] = T(double(u[id]) + (p1 - p0)); return; }
	const double phi0 = double(phi[c0]), phi1 = double(phi[c1]);
	if (phi0 <= 0 && phi1 <= 0) return;
	const double theta = phi0 / (phi0 - phi1);
	const double coef = 1 / fmax(phi0 <= 0 ? theta : 1 - theta, .001);
	u[id] = T(double(u[id]) + (p1 - p0) * coef);
}

// Copy the solve's statistics into the step record on the device.
__global__ void kRecordCg(const int *ints, const double *scal, const int *n, double *stats, const unsigned long long *counter) {
	double *rec = stepRecord(stats, counter);
	if (!rec) return;
	rec[kStUnknowns] = *n;
	rec[kStCgIters] = ints[0];
	rec[kStCgRefine] = ints[1];
	rec[kStCgResidual] = scal[0];
	rec[kStCgTol] = scal[1];
	rec[kStCgErr] = ints[4];
}

// Dynamic shared memory of a solve: the register form's matrix rows, kRegUnknowns slots of
// 2·dim entries per thread (98 KB mixed / 192 KB FP64 in 3D).
static size_t pcgRowBytes(bool mixed, int dim) {
	return size_t(kRegUnknowns) * size_t(2 * dim) * kCgBlock * (mixed ? sizeof(NbW32) : sizeof(NbW64));
}

// Lets the four solve kernels take their shared memory on the current device (above the
// 48 KB default); called before any capture.
garm_status pcgPrepare() {
	const struct { const void *fn; bool mixed; int dim; } k[4] = {
		{(const void *)kPcgMixed<4>, true, 2}, {(const void *)kPcgMixed<6>, true, 3},
		{(const void *)kPcgFp64<4>, false, 2}, {(const void *)kPcgFp64<6>, false, 3}};
	for (const auto &q : k)
		if (cudaFuncSetAttribute(q.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(pcgRowBytes(q.mixed, q.dim))) != cudaSuccess) {
			cudaGetLastError();
			return GARM_CUDA_ERROR;
		}
	return GARM_OK;
}

template <int D, typename T>
garm_status projectAsync(State &s, bool record) {
	const unsigned nbC = gridFor(s.N);
	kUnknownFlags<D, T><<<nbC, kBlock, 0, s.stream>>>(s.geom, (const T *)s.phi, (const T *)s.fraction[0], (const T *)s.fraction[1], (const T *)s.fraction[2],
		s.grid2mat, s.scanBlock); s.launches++;
	GARM_CHECK_LAUNCH();
	kScanBlocks<<<1, 1024, 0, s.stream>>>(s.scanBlock, int(nbC), s.nUnknownsDev); s.launches++;
	GARM_CHECK_LAUNCH();
	kScatterUnknowns<<<nbC, kBlock, 0, s.stream>>>(s.N, s.scanBlock, s.grid2mat, s.mat2grid); s.launches++;
	GARM_CHECK_LAUNCH();

	BuildIO<D, T> bio{};
	bio.phi = (const T *)s.phi;
	for (int a = 0; a < 3; a++) { bio.fr[a] = (const T *)s.fraction[a]; bio.u[a] = (const T *)s.u[a]; bio.bv[a] = (const T *)s.bvel[a]; }
	bio.grid2mat = s.grid2mat;
	bio.ent = (NbW64 *)s.ent64; bio.diag = s.diag; bio.invd = s.invd; bio.rhs = s.rhs;
	bio.ent32 = s.mixed ? (NbW32 *)s.ent32 : nullptr; bio.diag32 = s.mixed ? s.diag32 : nullptr; bio.invd32 = s.mixed ? s.invd32 : nullptr;
	bio.hdr = s.rowHdr; bio.idx = s.rowIdx;
	bio.stride = s.N;
	kBuildSystem<D, T><<<nbC, kBlock, 0, s.stream>>>(s.geom, bio); s.launches++;
	GARM_CHECK_LAUNCH();

	CgArgs a{};
	a.nDev = s.nUnknownsDev;
	a.ent = (const NbW64 *)s.ent64; a.diag = s.diag; a.invd = s.invd;
	a.ent32 = (const NbW32 *)s.ent32; a.diag32 = s.diag32; a.invd32 = s.invd32;
	a.hdr = s.rowHdr; a.idx = s.rowIdx;
	a.stride = s.N;
	a.b = s.rhs;
	a.x = s.pres;
	a.r64 = s.cgR;
	a.p64 = s.cgP64; a.pack64[0] = s.cgPack[0]; a.pack64[1] = s.cgPack[1];
	a.e32 = s.cgE32; a.p32 = s.cgP32; a.pack32[0] = s.cgPack[0]; a.pack32[1] = s.cgPack[1];
	a.partials = s.partials; a.maxBlocks = s.maxBlocks;
	a.bar = s.barrier; a.err = s.cgInts + 4;
	a.tol = s.cfg.cg_tolerance; a.maxIter = s.cfg.cg_max_iters;
	a.drop = s.cfg.mixed_residual_drop; a.replaceEvery = s.cfg.mixed_replace_interval;
	a.scal = s.cgScalars; a.ints = s.cgInts;

	kClearWords<<<1, 32, 0, s.stream>>>(s.barrier, 2, (unsigned *)s.cgInts, 8); s.launches++;
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return GARM_CUDA_ERROR;

	void *kfn;
	if (s.mixed) kfn = (D == 2) ? (void *)kPcgMixed<4> : (void *)kPcgMixed<6>;
	else kfn = (D == 2) ? (void *)kPcgFp64<4> : (void *)kPcgFp64<6>;
	const size_t rowBytes = pcgRowBytes(s.mixed, D);
	int perSM = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kfn, kCgBlock, rowBytes);
	if (e != cudaSuccess || perSM <= 0) return GARM_CUDA_ERROR;
	// one resident 512-thread block per SM for large scenes; small scenes take one
	// block per cg_cells_per_block (default 4096) interior cells so that several
	// scenes' solves can share the GPU.  The cooperative launch verifies co-residency.
	int64_t interior = 1;
	for (int q = 0; q < D; q++) interior *= (s.geom.n[q] - 2 * s.geom.bw);
	const int64_t perBlock = s.cfg.cg_cells_per_block > 0 ? s.cfg.cg_cells_per_block : 4096;
	int blocks = int(std::min<int64_t>((interior + perBlock - 1) / perBlock, s.numSMs));
	if (blocks < 1) blocks = 1;
	if (blocks > s.maxBlocks) blocks = s.maxBlocks;
	void *args[] = {&a};
	e = cudaLaunchCooperativeKernel(kfn, dim3(blocks), dim3(kCgBlock), args, rowBytes, s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	s.launches++;

	kApplyPressure<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (T *)s.u[0], (T *)s.u[1], (T *)s.u[2], (const T *)s.phi, s.grid2mat, s.pres,
		s.F[0], s.F[1], s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();

	kRecordCg<<<1, 1, 0, s.stream>>>(s.cgInts, s.cgScalars, s.nUnknownsDev, record ? s.statsDev : nullptr, s.stepCounter); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// Statistics of the last solve (host readback; synchronises the stream).
garm_status projectStats(State &s, garm_step_stats *st) {
	int hi[8] = {}; double hs[2] = {}; int n = 0;
	cudaError_t e = cudaMemcpyAsync(hi, s.cgInts, sizeof(hi), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(hs, s.cgScalars, sizeof(hs), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&n, s.nUnknownsDev, sizeof(int), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	s.nUnknowns = n;
	if (st) {
		st->cg_iterations += hi[0];
		st->cg_refinements += hi[1];
		st->unknowns = n;
		st->cg_residual = hs[0];
	}
	if (hi[4]) return GARM_TIMEOUT;
	if (n > 0 && !(hs[0] <= hs[1])) return GARM_NOT_CONVERGED;
	return GARM_OK;
}

template <int D, typename T>
garm_status project(State &s, garm_step_stats *st) {
	GARM_TRY((projectAsync<D, T>(s, false)));
	return projectStats(s, st);
}

#define GARM_INST(D, T) template garm_status project<D, T>(State &, garm_step_stats *); template garm_status projectAsync<D, T>(State &, bool);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
