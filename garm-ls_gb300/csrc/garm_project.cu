// garm_project.cu — Projector::project (Source/Core/Projector.cpp:13-20) on the GPU.
//   setUnknowns          (Projector.cpp:125-156)  → flag + block scan + scatter: the same
//                                                   x-fastest numbering as the serial loop
//   buildLinearSystem    (Projector.cpp:30-68)    → matrix-free rows: diag, 2D neighbour ids/weights, rhs
//   solveLinearSystem    (Projector.cpp:158-163, LinearSystem.h:23-39)
//                        → one persistent cooperative Jacobi-PCG launch with FP64 dot products
//                          reduced in a fixed order (deterministic), two grid barriers per
//                          iteration; mixed mode wraps FP32 inner sweeps in FP64 iterative refinement
//   applyPressureGradient (Projector.cpp:91-123)
#include "garm_internal.h"

#include <cfloat>

namespace garm {

constexpr int kCgBlock = 512;
constexpr unsigned long long kBarrierSpinLimit = 20000000ull;  // x ~100 ns sleep: ~2 s, then GARM_TIMEOUT

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
	int *nbr;
	double *wts, *diag, *invd, *rhs;
	float *wts32, *diag32, *invd32;
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
		io.nbr[q * io.stride + r] = nb;
		io.wts[q * io.stride + r] = wt;
		if (io.wts32) io.wts32[q * io.stride + r] = float(wt);
	}
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
	const int *nbr;
	const double *w, *diag, *invd;
	const float *w32, *diag32, *invd32;
	int64_t stride;
	const double *b;
	double *x, *r, *z, *p0, *p1, *q;
	float *fr, *fz, *fp0, *fp1, *fq, *fe;
	double *partials;
	int maxBlocks;
	unsigned *bar;
	int *err;
	double tol;
	int maxIter;
	double innerTol;
	int maxRefine;
	double *scal;  // [0] relative residual, [1] tolerance used
	int *ints;     // [0] matvecs, [1] refinements
};

// Vectors written by other blocks in the previous phase.  gridSync() ends with
// fences of GPU scope, which order these plain (L1-cacheable) loads after the
// other blocks' stores; the read-only texture path (__ldg) is never used for them.
__device__ __forceinline__ double ldcg(const double *p) { return *p; }
__device__ __forceinline__ float ldcg(const float *p) { return *p; }

// Grid-wide barrier with a bounded wait.  Returns false when any block gave up.
__device__ bool gridSync(unsigned *bar, int *err) {
	__syncthreads();
	if (threadIdx.x == 0) {
		volatile unsigned *vgen = bar + 1;
		const unsigned gen = *vgen;
		__threadfence();
		const unsigned prev = atomicAdd(bar, 1u);
		if (prev == gridDim.x - 1) {
			atomicExch(bar, 0u);
			__threadfence();
			atomicAdd(bar + 1, 1u);
		} else {
			unsigned long long spins = 0;
			while (*vgen == gen) {
				__nanosleep(100);
				if (++spins > kBarrierSpinLimit) { atomicExch(err, 1); break; }
				if (*(volatile int *)err) break;
			}
		}
		__threadfence();
	}
	__syncthreads();
	return *(volatile int *)err == 0;
}

// Block partial sums of NV values → partials[v*maxBlocks + blockIdx]
template <int NV>
__device__ __forceinline__ void blockPartials(double (&acc)[NV], double *partials, int maxBlocks, double *sh) {
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
	for (int v = 0; v < NV; v++) {
		double x = warpSum(acc[v]);
		if (lane == 0) sh[v * 32 + w] = x;
	}
	__syncthreads();
	if (threadIdx.x < NV) {
		double s = 0;
		for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[threadIdx.x * 32 + q];
		partials[threadIdx.x * maxBlocks + blockIdx.x] = s;
	}
	__syncthreads();
}

// Sum of the gridDim partials of slot v, identical in every block (fixed lane
// partition and shuffle tree: deterministic).  Lane 0 then runs `fin` on the
// totals (scalar work done once per block) and the results are broadcast.
template <int NV, int NOUT, typename Fin>
__device__ __forceinline__ void gridTotals(const double *partials, int maxBlocks, double (&out)[NOUT], double *sh, Fin fin) {
	static_assert(NOUT >= NV, "outputs include the sums");
	const int lane = threadIdx.x & 31;
	if (threadIdx.x < 32) {
		double t[NOUT];
#pragma unroll
		for (int v = 0; v < NV; v++) {
			double s = 0;
			for (int b = lane; b < (int)gridDim.x; b += 32) s += ldcg(partials + v * maxBlocks + b);
			t[v] = warpSum(s);
		}
		if (lane == 0) {
			fin(t);
#pragma unroll
			for (int v = 0; v < NOUT; v++) sh[v] = t[v];
		}
	}
	__syncthreads();
#pragma unroll
	for (int v = 0; v < NOUT; v++) out[v] = sh[v];
	__syncthreads();
}

struct NoFin { __device__ void operator()(double *) const {} };

// Inner PCG over vectors of type V with the operator A_V = diag - Σ w·neighbour:
//   solve A e = rhs, e starts at 0.  Element-wise arithmetic is in V (FP32 in the
//   mixed form); each thread's partial dot product is promoted to FP64 and the
//   block and grid reductions run in FP64 in a fixed order; α and β are formed
//   in FP64 once per block.  Returns the number of matvecs; the final |r|^2 and
//   |rhs|^2 are left in *outRR / *outB2.
template <int NB, typename V>
__device__ int pcgCore(const CgArgs &a, int n, const V *w, const V *dg, const V *invd, const double *rhsD,
                       V *x, V *r, V *z, V *p0, V *p1, V *q, double tolRel, int maxIter, double *sh, double *outRR, double *outB2, bool *ok) {
	const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x, nthr = int64_t(gridDim.x) * blockDim.x;
	V acc0 = V(0), acc1 = V(0);
	for (int64_t i = tid; i < n; i += nthr) {
		const V bv = V(rhsD[i]);
		x[i] = V(0);
		r[i] = bv;
		const V zi = bv * invd[i];
		z[i] = zi;
		p0[i] = zi;
		acc0 = fma(bv, bv, acc0);
		acc1 = fma(bv, zi, acc1);
	}
	{
		double acc[2] = {double(acc0), double(acc1)};
		blockPartials<2>(acc, a.partials, a.maxBlocks, sh);
	}
	if (!gridSync(a.bar, a.err)) { *ok = false; return 0; }
	double tot[2];
	gridTotals<2, 2>(a.partials, a.maxBlocks, tot, sh, NoFin{});
	const double rhsNorm2 = tot[0];
	double rz = tot[1];
	*outB2 = rhsNorm2;
	*outRR = rhsNorm2;
	if (rhsNorm2 == 0) return 0;
	const double tol = fmax(tolRel, DBL_EPSILON / sqrt(rhsNorm2));
	const double threshold = fmax(tol * tol * rhsNorm2, DBL_MIN);
	if (rhsNorm2 < threshold) return 0;

	V *pc = p0, *po = p1;
	bool first = true;
	V beta = V(0);
	int it = 0;
	while (it < maxIter) {
		// Phase A: p' = z + beta p (first: p' = p0), q = A p', partial p'·q
		V pq = V(0);
		for (int64_t i = tid; i < n; i += nthr) {
			const V pi = first ? ldcg(pc + i) : fma(beta, ldcg(pc + i), ldcg(z + i));
			if (!first) po[i] = pi;
			V qi = dg[i] * pi;
#pragma unroll
			for (int k = 0; k < NB; k++) {
				const int nb = a.nbr[k * a.stride + i];
				if (nb >= 0) {
					const V pn = first ? ldcg(pc + nb) : fma(beta, ldcg(pc + nb), ldcg(z + nb));
					qi = fma(-w[k * a.stride + i], pn, qi);
				}
			}
			q[i] = qi;
			pq = fma(pi, qi, pq);
		}
		if (!first) { V *t = pc; pc = po; po = t; }
		first = false;
		double acc1[1] = {double(pq)};
		blockPartials<1>(acc1, a.partials, a.maxBlocks, sh);
		if (!gridSync(a.bar, a.err)) { *ok = false; return it; }
		double t1[1];
		const double rzc = rz;
		gridTotals<1, 1>(a.partials, a.maxBlocks, t1, sh, [rzc](double *t) { t[0] = rzc / t[0]; });  // α = rz / p·q
		const V alpha = V(t1[0]);
		// Phase B: x += alpha p; r -= alpha q; z = M^-1 r; partial r·r, r·z
		V rr = V(0), rzn = V(0);
		for (int64_t i = tid; i < n; i += nthr) {
			x[i] = fma(alpha, ldcg(pc + i), x[i]);
			const V ri = fma(-alpha, q[i], r[i]);
			r[i] = ri;
			const V zi = ri * invd[i];
			z[i] = zi;
			rr = fma(ri, ri, rr);
			rzn = fma(ri, zi, rzn);
		}
		double a2[2] = {double(rr), double(rzn)};
		blockPartials<2>(a2, a.partials, a.maxBlocks, sh);
		if (!gridSync(a.bar, a.err)) { *ok = false; return it + 1; }
		double t2[3];
		gridTotals<2, 3>(a.partials, a.maxBlocks, t2, sh, [rzc](double *u) { u[2] = u[1] / rzc; });  // β = rz_new / rz
		it++;
		*outRR = t2[0];
		if (t2[0] < threshold) break;
		beta = V(t2[2]);
		rz = t2[1];
	}
	return it;
}

// FP64 form: one PCG on the FP64 operator.
template <int NB>
__global__ void __launch_bounds__(kCgBlock) kPcgFp64(CgArgs a) {
	__shared__ double sh[2 * 32];
	const int n = *a.nDev;
	double rr = 0, b2 = 0;
	bool ok = true;
	const int mv = pcgCore<NB, double>(a, n, a.w, a.diag, a.invd, a.b, a.x, a.r, a.z, a.p0, a.p1, a.q, a.tol, a.maxIter, sh, &rr, &b2, &ok);
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		a.ints[0] = mv;
		a.ints[1] = 1;
		a.scal[0] = b2 > 0 ? sqrt(rr / b2) : 0;
		a.scal[1] = b2 > 0 ? fmax(a.tol, DBL_EPSILON / sqrt(b2)) : a.tol;
	}
}

// Mixed form: FP64 iterative refinement around FP32 inner PCG sweeps.
//   x64 = 0; repeat: r64 = b - A64 x64 (FP64); stop when |r64| <= tol |b|;
//   solve A32 e = r64 (FP32 vectors, FP64 dots) to innerTol; x64 += e.
template <int NB>
__global__ void __launch_bounds__(kCgBlock) kPcgMixed(CgArgs a) {
	__shared__ double sh[64];
	const int n = *a.nDev;
	const int64_t tid = int64_t(blockIdx.x) * blockDim.x + threadIdx.x, nthr = int64_t(gridDim.x) * blockDim.x;
	for (int64_t i = tid; i < n; i += nthr) a.x[i] = 0;
	int mvTotal = 0, sweeps = 0;
	double relres = 0, tolUsed = a.tol;
	for (;;) {
		// r64 = b - A64 x64 and |b|^2, |r64|^2 in FP64
		double acc[2] = {0, 0};
		for (int64_t i = tid; i < n; i += nthr) {
			double ax = a.diag[i] * ldcg(a.x + i);
#pragma unroll
			for (int k = 0; k < NB; k++) {
				const int nb = a.nbr[k * a.stride + i];
				if (nb >= 0) ax -= a.w[k * a.stride + i] * ldcg(a.x + nb);
			}
			const double bi = a.b[i];
			const double ri = bi - ax;
			a.r[i] = ri;
			acc[0] += bi * bi;
			acc[1] += ri * ri;
		}
		blockPartials<2>(acc, a.partials, a.maxBlocks, sh);
		if (!gridSync(a.bar, a.err)) break;
		double t[2];
		gridTotals<2, 2>(a.partials, a.maxBlocks, t, sh, NoFin{});
		if (t[0] == 0) { relres = 0; break; }
		tolUsed = fmax(a.tol, DBL_EPSILON / sqrt(t[0]));
		relres = sqrt(t[1] / t[0]);
		if (relres <= tolUsed || sweeps >= a.maxRefine) break;
		double rr = 0, b2 = 0;
		bool ok = true;
		mvTotal += pcgCore<NB, float>(a, n, a.w32, a.diag32, a.invd32, a.r, a.fe, a.fr, a.fz, a.fp0, a.fp1, a.fq, a.innerTol, a.maxIter, sh, &rr, &b2, &ok);
		if (!ok) break;
		for (int64_t i = tid; i < n; i += nthr) a.x[i] += double(a.fe[i]);
		sweeps++;
		if (!gridSync(a.bar, a.err)) break;
	}
	if (blockIdx.x == 0 && threadIdx.x == 0) {
		a.ints[0] = mvTotal;
		a.ints[1] = sweeps;
		a.scal[0] = relres;
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

template <int D, typename T>
garm_status project(State &s, garm_step_stats *st) {
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
	bio.nbr = s.nbr; bio.wts = s.wts; bio.diag = s.diag; bio.invd = s.invd; bio.rhs = s.rhs;
	bio.wts32 = s.mixed ? s.wts32 : nullptr; bio.diag32 = s.mixed ? s.diag32 : nullptr; bio.invd32 = s.mixed ? s.invd32 : nullptr;
	bio.stride = s.N;
	kBuildSystem<D, T><<<nbC, kBlock, 0, s.stream>>>(s.geom, bio); s.launches++;
	GARM_CHECK_LAUNCH();

	CgArgs a{};
	a.nDev = s.nUnknownsDev;
	a.nbr = s.nbr; a.w = s.wts; a.diag = s.diag; a.invd = s.invd;
	a.w32 = s.wts32; a.diag32 = s.diag32; a.invd32 = s.invd32;
	a.stride = s.N;
	a.b = s.rhs;
	a.x = s.pres; a.r = s.cgR; a.z = s.cgZ; a.p0 = s.cgP0; a.p1 = s.cgP1; a.q = s.cgQ;
	a.fr = s.fR; a.fz = s.fZ; a.fp0 = s.fP0; a.fp1 = s.fP1; a.fq = s.fQ; a.fe = s.fE;
	a.partials = s.partials; a.maxBlocks = s.maxBlocks;
	a.bar = s.barrier; a.err = s.cgInts + 4;
	a.tol = s.cfg.cg_tolerance; a.maxIter = s.cfg.cg_max_iters;
	a.innerTol = s.cfg.mixed_inner_tolerance; a.maxRefine = s.cfg.mixed_max_refinements;
	a.scal = s.cgScalars; a.ints = s.cgInts;

	cudaError_t e = cudaMemsetAsync(s.barrier, 0, 2 * sizeof(unsigned), s.stream);
	if (e == cudaSuccess) e = cudaMemsetAsync(s.cgInts, 0, 8 * sizeof(int), s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;

	void *kfn;
	if (s.mixed) kfn = (D == 2) ? (void *)kPcgMixed<4> : (void *)kPcgMixed<6>;
	else kfn = (D == 2) ? (void *)kPcgFp64<4> : (void *)kPcgFp64<6>;
	int perSM = 0;
	e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, kfn, kCgBlock, 0);
	if (e != cudaSuccess || perSM <= 0) return GARM_CUDA_ERROR;
	int blocks = s.numSMs;  // one resident block per SM (occupancy permitting)
	if (perSM < 1) return GARM_CUDA_ERROR;
	if (blocks > s.maxBlocks) blocks = s.maxBlocks;
	void *args[] = {&a};
	e = cudaLaunchCooperativeKernel(kfn, dim3(blocks), dim3(kCgBlock), args, 0, s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	s.launches++;

	kApplyPressure<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (T *)s.u[0], (T *)s.u[1], (T *)s.u[2], (const T *)s.phi, s.grid2mat, s.pres,
		s.F[0], s.F[1], s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();

	int hi[8] = {}; double hs[2] = {}; int n = 0;
	e = cudaMemcpyAsync(hi, s.cgInts, sizeof(hi), cudaMemcpyDeviceToHost, s.stream);
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

#define GARM_INST(D, T) template garm_status project<D, T>(State &, garm_step_stats *);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
