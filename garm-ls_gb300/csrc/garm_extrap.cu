// garm_extrap.cu — boundary set-up, extrapolation, body force, wall condition, max |u|.
//   Boundary::reset/finish/getFaceFraction   (Source/Core/Boundary.cpp:19-35, 79-87, 135-174)
//   Extrapolation::solve (cell double / uchar / VectorDd / face)  (Source/Core/Extrapolation.h:42-218)
//   extrapolateFieldsToCollider              (Source/Core/LevelSetLiquid.cpp:1086-1137)
//   extrapolateFieldsToAir                   (LevelSetLiquid.cpp:1059-1084)
//   applyBodyForces (gravity)                (LevelSetLiquid.cpp:837-841)
//   Boundary::enforce(SGridBasedData)        (Boundary.cpp:89-120)
//   GridBasedData::normMax                   (Source/Core/GridBasedData.h:55-68)
#include "garm_internal.h"

#include <algorithm>

namespace garm {

// ---------------------------------------------------------------------------
// Boundary set-up — FP64 with explicit rounding so that face fractions and
// their thresholds (> .9, <= 0) match the host computation exactly.
// ---------------------------------------------------------------------------
template <int D>
struct BoxDev {
	double c[3], h[3];
	// ImplicitBox::signedDistance (Source/Core/ImplicitSurface.h:51-56)
	__device__ double sd(const double *p) const {
		double phi[3]; bool allIn = true;
		for (int i = 0; i < D; i++) { phi[i] = __dsub_rn(fabs(__dsub_rn(p[i], c[i])), h[i]); if (!(phi[i] <= 0)) allIn = false; }
		if (allIn) { double m = phi[0]; for (int i = 1; i < D; i++) if (phi[i] > m) m = phi[i]; return m; }
		double s = 0;
		for (int i = 0; i < D; i++) { const double q = fmax(phi[i], 0.0); s = __dadd_rn(s, __dmul_rn(q, q)); }
		return sqrt(s);
	}
	// ImplicitBox::closestNormal (ImplicitSurface.h:38-49), component `a`
	__device__ double normal(const double *p, int a) const {
		double phi[3], n[3]; bool allIn = true;
		for (int i = 0; i < D; i++) { phi[i] = __dsub_rn(fabs(__dsub_rn(p[i], c[i])), h[i]); if (!(phi[i] <= 0)) allIn = false; }
		if (allIn) {
			int ax = 0; for (int i = 1; i < D; i++) if (phi[i] > phi[ax]) ax = i;
			for (int i = 0; i < D; i++) n[i] = (i == ax) ? 1.0 : 0.0;
		} else for (int i = 0; i < D; i++) n[i] = fmax(phi[i], 0.0);
		double z = 0;
		for (int i = 0; i < D; i++) {
			const double d = __dsub_rn(p[i], c[i]);
			const double sg = d > 0 ? 1.0 : (d < 0 ? -1.0 : 0.0);
			n[i] = __dmul_rn(n[i], sg);
			z = __dadd_rn(z, __dmul_rn(n[i], n[i]));
		}
		if (z > 0) return n[a] / sqrt(z);
		return n[a];
	}
};

template <int D>
static BoxDev<D> domainBox(const Geom &g) {
	BoxDev<D> b{};
	for (int i = 0; i < D; i++) {
		const double minC = g.o[i] + 1.0 * g.bw * g.dx;                  // StaggeredGrid::domainOrigin
		const double len = double(g.n[i] - 1 * g.bw * 2) * g.dx;        // StaggeredGrid::domainLengths
		b.c[i] = minC + len / 2;
		b.h[i] = len / 2;
	}
	return b;
}

template <int D, typename T>
__global__ void kBoundaryReset(Geom geom, BoxDev<D> box, double *nodeDist, T *cellDist, T *fr0, T *fr1, T *fr2, T *n0, T *n1, T *n2,
                               int64_t NN, int64_t N, int64_t F0, int64_t F1, int64_t Ftot) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id < NN) {
		const G<D, double> g = nodeGrid<D, double>(geom);
		int i, j, k; g.coord(id, i, j, k);
		const double p[3] = {g.pos(0, i), g.pos(1, j), D == 3 ? g.pos(2, k) : 0.0};
		nodeDist[id] = -box.sd(p);
		return;
	}
	id -= NN;
	if (id < N) {
		const G<D, double> g = cellGrid<D, double>(geom);
		int i, j, k; g.coord(id, i, j, k);
		const double p[3] = {g.pos(0, i), g.pos(1, j), D == 3 ? g.pos(2, k) : 0.0};
		cellDist[id] = T(-box.sd(p));
		return;
	}
	id -= N;
	if (id >= Ftot) return;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, double> g = faceGrid<D, double>(geom, axis);
	int i, j, k; g.coord(id, i, j, k);
	const double p[3] = {g.pos(0, i), g.pos(1, j), D == 3 ? g.pos(2, k) : 0.0};
	T *fr = axis == 0 ? fr0 : (axis == 1 ? fr1 : fr2);
	T *nr = axis == 0 ? n0 : (axis == 1 ? n1 : n2);
	fr[id] = T(-box.sd(p));
	nr[id] = T(-box.normal(p, axis));
}

// Boundary::finish → getFaceFraction (Boundary.cpp:79-87, 135-174)
template <int D, typename T>
__global__ void kBoundaryFinish(Geom geom, const double *nodeDist, T *fr0, T *fr1, T *fr2, int64_t F0, int64_t F1, int64_t Ftot) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, double> g = faceGrid<D, double>(geom, axis);
	const G<D, double> ng = nodeGrid<D, double>(geom);
	int f[3]; g.coord(id, f[0], f[1], f[2]);
	T *fr = axis == 0 ? fr0 : (axis == 1 ? fr1 : fr2);
	// StaggeredGrid::isBoundaryFace (StaggeredGrid.h:57)
	bool inside = true;
	for (int a = 0; a < D; a++) if (f[a] < geom.bw || f[a] >= g.s[a] - geom.bw) inside = false;
	if (f[axis] <= geom.bw || f[axis] >= geom.n[axis] - geom.bw || !inside) { fr[id] = T(1); return; }
	auto theta = [](double p0, double p1) { return p0 / __dsub_rn(p0, p1); };
	double ff;
	if (D == 2) {
		int n0[3] = {f[0], f[1], 0}, n1[3] = {f[0], f[1], 0};
		n1[axis ^ 1] += 1;
		const double p0 = nodeDist[ng.idx(n0[0], n0[1], 0)], p1 = nodeDist[ng.idx(n1[0], n1[1], 0)];
		if (p0 <= 0 && p1 <= 0) ff = 1;
		else if (p0 <= 0 && p1 > 0) ff = theta(p0, p1);
		else if (p0 > 0 && p1 <= 0) ff = theta(p1, p0);
		else ff = 0;
	} else {
		const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
		double p[4];
		for (int o = 0; o < 4; o++) {
			int n[3] = {f[0], f[1], f[2]};
			n[a1] += (o & 1); n[a2] += (o >> 1 & 1);
			p[o] = nodeDist[ng.idx(n[0], n[1], n[2])];
		}
		auto fr3 = [&](double q0, double q1, double q2) -> double {
			double t;
			if (q0 > q1) { t = q0; q0 = q1; q1 = t; }
			if (q1 > q2) { t = q1; q1 = q2; q2 = t; }
			if (q0 > q1) { t = q0; q0 = q1; q1 = t; }
			if (q2 <= 0) return 1;
			else if (q1 <= 0) return __dsub_rn(1.0, __dmul_rn(theta(q2, q0), theta(q2, q1)));
			else if (q0 <= 0) return __dmul_rn(theta(q0, q1), theta(q0, q2));
			else return 0;
		};
		const double c = __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(p[0], p[1]), p[2]), p[3]), .25);
		ff = __dmul_rn(__dadd_rn(__dadd_rn(__dadd_rn(fr3(c, p[0], p[1]), fr3(c, p[1], p[3])), fr3(c, p[3], p[2])), fr3(c, p[2], p[0])), .25);
	}
	fr[id] = T(ff > .9 ? 1.0 : ff);
}

// Work list of faces that Boundary::enforce touches (fraction > 0.1).
template <int D, typename T>
__global__ void kCollectBcFaces(const T *fr0, const T *fr1, const T *fr2, int64_t F0, int64_t F1, int64_t Ftot, int64_t *list, int *count) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	const int64_t gid = id;
	const T *fr = fr0;
	if (id >= F0) { id -= F0; fr = fr1; if (id >= F1) { id -= F1; fr = fr2; } }
	const T v = fr[id];
	if (v > T(0.1) && v <= T(1)) list[atomicAdd(count, 1)] = gid;
}

template <int D, typename T>
garm_status initBoundary(State &s) {
	const BoxDev<D> box = domainBox<D>(s.geom);
	const int64_t total = s.NN + s.N + s.Ftot;
	kBoundaryReset<D, T><<<gridFor(total), kBlock, 0, s.stream>>>(s.geom, box, (double *)s.nodeDist, (T *)s.cellDist,
		(T *)s.fraction[0], (T *)s.fraction[1], (T *)s.fraction[2], (T *)s.normal[0], (T *)s.normal[1], (T *)s.normal[2],
		s.NN, s.N, s.F[0], s.F[1], s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status finishBoundary(State &s) {
	kBoundaryFinish<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (const double *)s.nodeDist,
		(T *)s.fraction[0], (T *)s.fraction[1], (T *)s.fraction[2], s.F[0], s.F[1], s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();
	cudaError_t e = cudaMemsetAsync(s.redI32, 0, sizeof(int), s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	kCollectBcFaces<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>((const T *)s.fraction[0], (const T *)s.fraction[1], (const T *)s.fraction[2],
		s.F[0], s.F[1], s.Ftot, s.bcList, s.redI32); s.launches++;
	GARM_CHECK_LAUNCH();
	int n = 0;
	e = cudaMemcpyAsync(&n, s.redI32, sizeof(int), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	s.nBc = n;
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// Extrapolation (Extrapolation.h:42-218) as a frontier march.
//
// The reference runs maxSteps Jacobi passes over the whole grid.  In pass p, every cell
// outside the visited set that has a visited neighbour becomes the mean of its visited
// neighbours, taken in the order -x,+x,-y,+y,-z,+z (Grid.h:59-60), and joins the set.  The
// cells that change in pass p are exactly the unvisited neighbours of the cells that joined
// in pass p-1 (of the seeds, for p = 1).  So one cooperative launch keeps that frontier as
// a list and touches only it:
//   phase A (all elements): seed levels, and the final value of elements that may never be
//           reached (ξ = x, u = 0, advRegion = 0); those values are never read before the
//           element joins and overwrites them;
//   phase B (all elements): the first frontier, the unvisited neighbours of seeds;
//   pass p (one small launch over the frontier): each frontier element takes the mean of
//           its neighbours with level < p, sets its level to p and queues its unvisited
//           neighbours (each element once, by a bit claimed with atomicOr) as the frontier
//           of pass p+1.
// level = 0 for seeds, p for elements that joined in pass p, 255 otherwise.  A pass reads
// only neighbours with level < p, which no thread of that pass writes, so the passes keep
// the reference's Jacobi semantics; the values and the summation order are the reference's,
// and the result does not depend on the list order.
// ---------------------------------------------------------------------------
enum FrontKind { kFrontCollider = 0, kFrontRefMap = 1, kFrontAdv = 2, kFrontFaces = 3 };

constexpr int kFrontElemsPerBlock = 4096;   // grid elements per block of the pass launches (at most 8 blocks per SM)

template <typename T>
struct FrontArgs {
	Geom geom;
	int nsub;              // sub-grids: 1 (cells) or D (face grids)
	int off[4];            // first element of each sub-grid (off[nsub] = total)
	int size[3][3];        // sub-grid sizes
	T *val[3];             // collider: ori, φ; reference map: ξ components; faces: u per axis
	uint8_t *flag;         // advRegion
	const T *cellDist, *ori, *fr[3];
	const uint8_t *adv;
	uint8_t *level;
	unsigned *bits;        // queued-once bits, one per element
	int *list[2];          // frontier of pass p in list[p & 1]
	int *count;            // [p]: frontier size of pass p
	int passes;
};

struct FrontPos { int sub, local, i, j, k; };

template <int D, typename T>
__device__ __forceinline__ FrontPos frontPos(const FrontArgs<T> &a, int gid) {
	FrontPos p;
	p.sub = 0;
	if (a.nsub > 1 && gid >= a.off[1]) p.sub = (a.nsub > 2 && gid >= a.off[2]) ? 2 : 1;
	p.local = gid - a.off[p.sub];
	const unsigned sx = unsigned(a.size[p.sub][0]), r = unsigned(p.local) / sx;
	p.i = p.local - int(r * sx);
	if (D == 2) { p.j = int(r); p.k = 0; }
	else { const unsigned sy = unsigned(a.size[p.sub][1]); const unsigned q = r / sy; p.j = int(r - q * sy); p.k = int(q); }
	return p;
}

// Neighbour q (-x,+x,-y,+y,-z,+z) of an element in its own sub-grid, or -1 outside it.
template <int D, typename T>
__device__ __forceinline__ int frontNeighbour(const FrontArgs<T> &a, const FrontPos &p, int gid, int q) {
	const int sx = a.size[p.sub][0], sy = a.size[p.sub][1], sz = D == 3 ? a.size[p.sub][2] : 1;
	switch (q) {
	case 0: return p.i > 0 ? gid - 1 : -1;
	case 1: return p.i < sx - 1 ? gid + 1 : -1;
	case 2: return p.j > 0 ? gid - sx : -1;
	case 3: return p.j < sy - 1 ? gid + sx : -1;
	case 4: return p.k > 0 ? gid - sx * sy : -1;
	default: return p.k < sz - 1 ? gid + sx * sy : -1;
	}
}

__device__ __forceinline__ uint8_t ldLevel(const uint8_t *p) { return *(const volatile uint8_t *)p; }

// Claims element `nb` for the next frontier; true when this thread set its bit.
__device__ __forceinline__ bool claim(unsigned *bits, int nb) {
	const unsigned m = 1u << (nb & 31);
	return (atomicOr(bits + (nb >> 5), m) & m) == 0;
}

// Seed test of a face: a liquid face of extrapolateFieldsToAir (LevelSetLiquid.cpp:1074-1082),
// fraction < 1 and the level set <= 0 in one of the two cells beside it.
template <int D, typename T>
__device__ __forceinline__ bool liquidFace(const FrontArgs<T> &a, const FrontPos &p) {
	if (!(a.fr[p.sub][p.local] < T(1))) return false;
	const G<D, T> cg = cellGrid<D, T>(a.geom);
	const int axis = p.sub;
	const int i0 = p.i - (axis == 0), j0 = p.j - (axis == 1), k0 = p.k - (axis == 2);
	if (!cg.valid(p.i, p.j, p.k) || !cg.valid(i0, j0, k0)) return false;  // never for interior faces (fraction < 1)
	return a.ori[cg.idx(i0, j0, k0)] <= T(0) || a.ori[cg.idx(p.i, p.j, p.k)] <= T(0);
}

// Phase A: levels and the values of elements that may never be reached; the queued bits
// and the frontier sizes start at zero (kernel stores, not memset nodes, which serialise
// concurrent scenes' graphs).
template <int D, typename T, int Kind>
__global__ void __launch_bounds__(kBlock) kFrontSeed(FrontArgs<T> a, const int *gate) {
	pdlWait();
	if (gate && !*gate) return;
	const int gid = int(blockIdx.x) * blockDim.x + threadIdx.x;
	if (gid < (a.off[a.nsub] + 31) / 32) a.bits[gid] = 0u;
	if (gid < a.passes + 2) a.count[gid] = 0;
	if (gid >= a.off[a.nsub]) return;
	bool seed;
	if (Kind == kFrontCollider) seed = a.cellDist[gid] > T(0);
	else if (Kind == kFrontRefMap) {
		seed = a.adv[gid] > 0;
		if (!seed) {
			const FrontPos p = frontPos<D, T>(a, gid);
			const G<D, T> g = cellGrid<D, T>(a.geom);
			a.val[0][gid] = g.pos(0, p.i); a.val[1][gid] = g.pos(1, p.j); if (D == 3) a.val[2][gid] = g.pos(2, p.k);
		}
	} else if (Kind == kFrontAdv) {
		seed = a.ori[gid] <= T(0);
		a.flag[gid] = seed ? 1 : 0;
	} else {
		const FrontPos p = frontPos<D, T>(a, gid);
		seed = liquidFace<D, T>(a, p);
		if (!seed) a.val[p.sub][p.local] = T(0);
	}
	a.level[gid] = seed ? 0 : 255;
}

// Phase B: the first frontier, the unvisited neighbours of seeds.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kFrontFirst(FrontArgs<T> a, const int *gate) {
	pdlWait();
	if (gate && !*gate) return;
	const int total = a.off[a.nsub];
	const int gid = int(blockIdx.x) * blockDim.x + threadIdx.x;
	int ids[1];
	int n = 0;
	if (gid < total && a.level[gid] == 255) {
		const FrontPos p = frontPos<D, T>(a, gid);
		bool touch = false;
#pragma unroll
		for (int q = 0; q < 2 * D; q++) {
			const int nb = frontNeighbour<D, T>(a, p, gid, q);
			if (nb >= 0 && a.level[nb] == 0) touch = true;
		}
		if (touch && claim(a.bits, gid)) ids[n++] = gid;
	}
	warpAppend(a.list[1], a.count + 1, ids, n);
}

// Pass `pass`: every element of its frontier joins; its unvisited neighbours form the next
// frontier.  A small grid strides over the frontier, whose size is on the device.
template <int D, typename T, int Kind>
__global__ void __launch_bounds__(kBlock) kFrontPass(FrontArgs<T> a, int pass, const int *gate) {
	pdlWait();
	if (gate && !*gate) return;
	const int stride = int(gridDim.x) * blockDim.x;
	const int n = a.count[pass];
	const int *cur = a.list[pass & 1];
	int *next = a.list[(pass + 1) & 1];
	for (int base = int(blockIdx.x) * blockDim.x; base < n; base += stride) {
		const int t = base + int(threadIdx.x);
		int ids[6];
		int m = 0;
		if (t < n) {
			const int gid = cur[t];
			const FrontPos p = frontPos<D, T>(a, gid);
			int nbs[6];
			int cnt = 0;
			T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
			for (int q = 0; q < 2 * D; q++) {
				nbs[q] = frontNeighbour<D, T>(a, p, gid, q);
				if (nbs[q] < 0 || ldLevel(a.level + nbs[q]) >= pass) continue;
				cnt++;
				if (Kind == kFrontCollider) { s0 += a.val[0][nbs[q]]; s1 += a.val[1][nbs[q]]; }
				else if (Kind == kFrontRefMap) { s0 += a.val[0][nbs[q]]; s1 += a.val[1][nbs[q]]; if (D == 3) s2 += a.val[2][nbs[q]]; }
				else if (Kind == kFrontFaces) s0 += a.val[p.sub][nbs[q] - a.off[p.sub]];
			}
			// cnt > 0: every frontier element neighbours an element that joined in the previous pass
			const T c = T(cnt);
			if (Kind == kFrontCollider) { a.val[0][gid] = s0 / c; a.val[1][gid] = s1 / c; }
			else if (Kind == kFrontRefMap) { a.val[0][gid] = s0 / c; a.val[1][gid] = s1 / c; if (D == 3) a.val[2][gid] = s2 / c; }
			else if (Kind == kFrontAdv) a.flag[gid] = 1;
			else a.val[p.sub][p.local] = s0 / c;
			*(volatile uint8_t *)(a.level + gid) = uint8_t(pass);
			if (pass < a.passes) {
#pragma unroll
				for (int q = 0; q < 2 * D; q++)
					if (nbs[q] >= 0 && ldLevel(a.level + nbs[q]) == 255 && claim(a.bits, nbs[q])) ids[m++] = nbs[q];
			}
		}
		warpAppend(next, a.count + pass + 1, ids, m);
	}
}

static inline int passCount(double r) { int n = 0; while (n < r) n++; return n; }  // `for (iter = 0; iter < maxSteps; ...)`

template <int D, typename T, int Kind>
static garm_status front(State &s, int passes, bool second = false) {
	cudaStream_t st = second ? s.aux : s.stream;
	FrontArgs<T> a{};
	a.geom = s.geom;
	if (Kind == kFrontFaces) {
		a.nsub = D;
		int o = 0;
		for (int ax = 0; ax < D; ax++) {
			a.off[ax] = o;
			for (int b = 0; b < 3; b++) a.size[ax][b] = s.geom.n[b] + (b == ax ? 1 : 0);
			if (D == 2) a.size[ax][2] = 1;
			o += int(s.F[ax]);
			a.val[ax] = (T *)s.u[ax];
			a.fr[ax] = (const T *)s.fraction[ax];
		}
		a.off[D] = o;
		a.level = s.fvis0;
	} else {
		a.nsub = 1;
		a.off[0] = 0;
		a.off[1] = int(s.N);
		for (int b = 0; b < 3; b++) a.size[0][b] = s.geom.n[b];
		if (D == 2) a.size[0][2] = 1;
		a.level = s.vis0;
		if (Kind == kFrontCollider) { a.val[0] = (T *)s.ori; a.val[1] = (T *)s.phi; }
		if (Kind == kFrontRefMap) for (int c = 0; c < D; c++) a.val[c] = (T *)s.xi[c];
	}
	a.flag = s.adv;
	a.adv = s.adv;
	a.cellDist = (const T *)s.cellDist;
	a.ori = (const T *)s.ori;
	a.bits = second ? s.frontBitsB : s.frontBits;
	a.list[0] = second ? s.frontListB[0] : s.frontList[0];
	a.list[1] = second ? s.frontListB[1] : s.frontList[1];
	a.count = second ? s.frontCountB : s.frontCount;
	a.passes = passes;
	if (passes > kFrontMaxPasses) return GARM_INVALID;
	const int total = a.off[a.nsub];
	const int *gate = s.gate;
	launchPdl(kFrontSeed<D, T, Kind>, dim3(gridFor(total)), dim3(kBlock), st, a, gate); s.launches++;
	GARM_CHECK_LAUNCH();
	if (passes <= 0) return GARM_OK;
	launchPdl(kFrontFirst<D, T>, dim3(gridFor(total)), dim3(kBlock), st, a, gate); s.launches++;
	GARM_CHECK_LAUNCH();
	// the frontiers are thin shells: a grid in proportion to the grid size, at most 8 blocks
	// per SM, enough warps to hide the latency of the scattered shell
	const unsigned blocks = unsigned(std::max<int64_t>(1, std::min<int64_t>((int64_t(total) + kFrontElemsPerBlock - 1) / kFrontElemsPerBlock, 8 * int64_t(s.numSMs))));
	for (int pass = 1; pass <= passes; pass++) {
		launchPdl(kFrontPass<D, T, Kind>, dim3(blocks), dim3(kBlock), st, a, pass, gate); s.launches++;
	}
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// extrapolateFieldsToCollider (LevelSetLiquid.cpp:1086-1117): ori and φ from cellDist > 0.
template <int D, typename T>
garm_status extrapolateToCollider(State &s) {
	return front<D, T, kFrontCollider>(s, passCount(s.cfg.boundary_extrap_radius));
}

// extrapolateFieldsToAir (LevelSetLiquid.cpp:1059-1084): ξ from advRegion > 0 (unreached
// cells get ξ = x); advRegion = (ori <= 0) dilated (unreached cells 0); u from the liquid
// faces over airExtrapolationRadius + 2 passes (unreached faces 0).
template <int D, typename T>
garm_status extrapolateToAir(State &s) {
	const int R = passCount(s.cfg.air_extrap_radius);
	// the face march reads ori and the fractions only, so it runs beside the two cell
	// marches (ξ, then the flags, which ξ's seeds are read from) on the second stream
	GARM_TRY(forkAux(s, 1));
	GARM_TRY((front<D, T, kFrontFaces>(s, passCount(s.cfg.air_extrap_radius + 2), true)));
	GARM_TRY((front<D, T, kFrontRefMap>(s, R)));
	GARM_TRY((front<D, T, kFrontAdv>(s, R)));
	return joinAux(s, 1);
}

// ---------------------------------------------------------------------------
// Body force: u_y -= 9.8 dt on every y-face
// ---------------------------------------------------------------------------
template <typename T>
__global__ void kGravity(int64_t n, T *u, const double *dtp) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id < n) u[id] -= T(9.8 * *dtp);  // kGravity * dt (Constants.h:9)
}

template <int D, typename T>
garm_status bodyForce(State &s) {
	if (!s.cfg.enable_gravity) return GARM_OK;
	kGravity<T><<<gridFor(s.F[1]), kBlock, 0, s.stream>>>(s.F[1], (T *)s.u[1], s.dtDev); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// Boundary::enforce(u) over the fraction > 0.1 work list: compute, then scatter.
// ---------------------------------------------------------------------------
template <int D, typename T>
struct SVec { const T *p[3]; };

template <int D, typename T>
__global__ void kEnforceBc(Geom geom, const int64_t *list, int64_t nList, SVec<D, T> u, SVec<D, T> nrm, SVec<D, T> bv, const T *fr0, const T *fr1, const T *fr2,
                           int64_t F0, int64_t F1, T *out) {
	const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= nList) return;
	int64_t id = list[t];
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, T> g = faceGrid<D, T>(geom, axis);
	G<D, T> fg[3];
	for (int a = 0; a < D; a++) fg[a] = faceGrid<D, T>(geom, a);
	int i, j, k; g.coord(id, i, j, k);
	const T pos[3] = {g.pos(0, i), g.pos(1, j), D == 3 ? g.pos(2, k) : T(0)};
	const T *uu = u.p[axis];
	T n[3] = {T(0), T(0), T(0)};
	for (int a = 0; a < D; a++) n[a] = lerp<D, T>(nrm.p[a], fg[a], pos);
	T z = T(0);
	for (int a = 0; a < D; a++) z += n[a] * n[a];
	if (z > T(0)) { const T r = sqrt(z); for (int a = 0; a < D; a++) n[a] = n[a] / r; }
	bool any = false;
	for (int a = 0; a < D; a++) if (n[a] != T(0)) any = true;
	T res = uu[id];
	if (any) {
		T vel[3] = {T(0), T(0), T(0)}, vel0[3] = {T(0), T(0), T(0)};
		for (int a = 0; a < D; a++) { vel[a] = lerp<D, T>(u.p[a], fg[a], pos); vel0[a] = lerp<D, T>(bv.p[a], fg[a], pos); }
		T vn = T(0);
		for (int a = 0; a < D; a++) vn += (vel[a] - vel0[a]) * n[a];
		if (vn < T(0)) {
			const T vt = (vel[axis] - vel0[axis]) - vn * n[axis];
			res = (vel[axis] - vn * n[axis]) - T(0.8) * vt;
		}
	}
	out[t] = res;
}

template <typename T>
__global__ void kScatterBc(const int64_t *list, int64_t nList, const T *vals, T *u0, T *u1, T *u2, int64_t F0, int64_t F1) {
	const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (t >= nList) return;
	int64_t id = list[t];
	T *u = u0;
	if (id >= F0) { id -= F0; u = u1; if (id >= F1) { id -= F1; u = u2; } }
	u[id] = vals[t];
}

template <int D, typename T>
garm_status enforceBoundaryConditions(State &s) {
	if (s.nBc == 0) return GARM_OK;
	SVec<D, T> u{}, nr{}, bv{};
	for (int a = 0; a < 3; a++) { u.p[a] = (const T *)s.u[a]; nr.p[a] = (const T *)s.normal[a]; bv.p[a] = (const T *)s.bvel[a]; }
	kEnforceBc<D, T><<<gridFor(s.nBc), kBlock, 0, s.stream>>>(s.geom, s.bcList, s.nBc, u, nr, bv, (const T *)s.fraction[0], (const T *)s.fraction[1],
		(const T *)s.fraction[2], s.F[0], s.F[1], (T *)s.bcTmp); s.launches++;
	GARM_CHECK_LAUNCH();
	kScatterBc<T><<<gridFor(s.nBc), kBlock, 0, s.stream>>>(s.bcList, s.nBc, (const T *)s.bcTmp, (T *)s.u[0], (T *)s.u[1], (T *)s.u[2], s.F[0], s.F[1]); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// max |u| over all faces.  Non-negative doubles order like their bit patterns,
// so an integer atomicMax gives a deterministic result.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBlock) kMaxAbs(const T *u0, const T *u1, const T *u2, int64_t F0, int64_t F1, int64_t Ftot, unsigned long long *out) {
	double m = 0;
	for (int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; id < Ftot; id += int64_t(gridDim.x) * blockDim.x) {
		int64_t q = id; const T *u = u0;
		if (q >= F0) { q -= F0; u = u1; if (q >= F1) { q -= F1; u = u2; } }
		m = fmax(m, fabs(double(u[q])));
	}
	for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
	__shared__ double sh[kBlock / 32];
	if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int q = 1; q < kBlock / 32; q++) m = fmax(m, sh[q]);
		atomicMax(out, (unsigned long long)__double_as_longlong(m));
	}
}

// dt of the next step from max|u| on the device: stepRate*dx/max|u| (LevelSetLiquid.h:129)
// clamped to the end of the frame and halved when two steps remain (Simulator.cpp:110-117).
// clock = {time within the frame, frame length, cfl}.
__global__ void kStepDt(const unsigned long long *maxBits, double dx, double *clock, double *dt, double *stats, const unsigned long long *counter) {
	double *rec = stepRecord(stats, counter);
	const double m = __longlong_as_double((long long)*maxBits);
	const double target = clock[1];
	double time = clock[0];
	double d = clock[2] * dx / m;  // +inf at rest, as the reference
	if (time + d >= target) { d = target - time; time = 0; }
	else { if (time + 2 * d >= target) d = (target - time) / 2; time += d; }
	clock[0] = time;
	*dt = d;
	if (rec) rec[kStDt] = d;
}

__global__ void kClearWords(unsigned *a, int na, unsigned *b, int nb) {
	const int t = int(threadIdx.x);
	if (t < na) a[t] = 0u;
	if (t < nb) b[t] = 0u;
}

template <int D, typename T>
garm_status maxSpeedAsync(State &s) {
	kClearWords<<<1, 32, 0, s.stream>>>((unsigned *)s.redU64, 2, nullptr, 0); s.launches++;
	const unsigned nb = unsigned(s.numSMs > 0 ? s.numSMs * 8 : 1024);
	kMaxAbs<T><<<nb, kBlock, 0, s.stream>>>((const T *)s.u[0], (const T *)s.u[1], (const T *)(D == 3 ? s.u[2] : s.u[0]), s.F[0], s.F[1], s.Ftot, s.redU64); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status maxSpeed(State &s, double *out) {
	cudaError_t e = cudaMemsetAsync(s.redU64, 0, sizeof(unsigned long long), s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	const unsigned nb = unsigned(s.numSMs > 0 ? s.numSMs * 8 : 1024);
	kMaxAbs<T><<<nb, kBlock, 0, s.stream>>>((const T *)s.u[0], (const T *)s.u[1], (const T *)(D == 3 ? s.u[2] : s.u[0]), s.F[0], s.F[1], s.Ftot, s.redU64); s.launches++;
	GARM_CHECK_LAUNCH();
	unsigned long long bits = 0;
	e = cudaMemcpyAsync(&bits, s.redU64, sizeof(bits), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	double m;
	static_assert(sizeof(m) == sizeof(bits), "size");
	memcpy(&m, &bits, sizeof(m));
	*out = m;
	return GARM_OK;
}

template <typename T>
__global__ void kCopy(int64_t n, T *dst, const T *src) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id < n) dst[id] = src[id];
}

template <int D, typename T>
garm_status copyField(State &s, void *dst, const void *src, int64_t n) {
	kCopy<T><<<gridFor(n), kBlock, 0, s.stream>>>(n, (T *)dst, (const T *)src); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

#define GARM_INST(D, T) \
	template garm_status initBoundary<D, T>(State &); \
	template garm_status finishBoundary<D, T>(State &); \
	template garm_status extrapolateToCollider<D, T>(State &); \
	template garm_status extrapolateToAir<D, T>(State &); \
	template garm_status bodyForce<D, T>(State &); \
	template garm_status enforceBoundaryConditions<D, T>(State &); \
	template garm_status maxSpeed<D, T>(State &, double *); \
	template garm_status maxSpeedAsync<D, T>(State &); \
	template garm_status copyField<D, T>(State &, void *, const void *, int64_t);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
