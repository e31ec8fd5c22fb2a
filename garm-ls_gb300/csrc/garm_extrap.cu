// garm_extrap.cu — boundary set-up, extrapolation, body force, wall condition, max |u|.
//   Boundary::reset/finish/getFaceFraction   (Source/Core/Boundary.cpp:19-35, 79-87, 135-174)
//   Extrapolation::solve (cell double / uchar / VectorDd / face)  (Source/Core/Extrapolation.h:42-218)
//   extrapolateFieldsToCollider              (Source/Core/LevelSetLiquid.cpp:1086-1137)
//   extrapolateFieldsToAir                   (LevelSetLiquid.cpp:1059-1084)
//   applyBodyForces (gravity)                (LevelSetLiquid.cpp:837-841)
//   Boundary::enforce(SGridBasedData)        (Boundary.cpp:89-120)
//   GridBasedData::normMax                   (Source/Core/GridBasedData.h:55-68)
#include "garm_internal.h"

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
// Extrapolation passes.  Values are updated in place: a pass reads only cells
// already in the visited set and writes only cells outside it, so it has the
// reference's Jacobi semantics; the visited mask is double-buffered.
// ---------------------------------------------------------------------------
enum FixedKind { kFixedCellDistPos = 0, kFixedAdvPos = 1, kFixedOriNonPos = 2 };

template <typename T>
__global__ void kCellMask(int64_t N, int kind, const T *cellDist, const uint8_t *adv, const T *ori, uint8_t *vis, const int *gate) {
	if (gate && !*gate) return;
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= N) return;
	bool f;
	if (kind == kFixedCellDistPos) f = cellDist[id] > T(0);
	else if (kind == kFixedAdvPos) f = adv[id] > 0;
	else f = ori[id] <= T(0);
	vis[id] = f ? 1 : 0;
}

// Kind 0: NS scalar planes (cell double, Extrapolation.h:86-126)
// Kind 1: D-vector reference map; unreached cells get their position (Extrapolation.h:176-218)
// Kind 2: flag (uchar) (Extrapolation.h:128-174)
// Neighbours are visited in the reference's order -x,+x,-y,+y,-z,+z (Grid.h:59-60).
template <int D, typename T, int Kind, int NS>
__global__ void __launch_bounds__(kBlock) kExtrapCellPass(Geom geom, T *f0, T *f1, T *f2, uint8_t *flag, const uint8_t *__restrict__ vis0, uint8_t *vis1, const int *gate) {
	if (gate && !*gate) return;
	const int sx = geom.n[0], sy = geom.n[1], sz = D == 3 ? geom.n[2] : 1;
	const int N = sx * sy * sz;
	const int id = int(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= N) return;
	if (vis0[id]) { vis1[id] = 1; return; }
	const unsigned r = unsigned(id) / unsigned(sx);
	const int i = id - int(r) * sx;
	const int j = D == 3 ? int(r % unsigned(sy)) : int(r);
	const int k = D == 3 ? int(r / unsigned(sy)) : 0;
	const int sxy = sx * sy;
	const int off[6] = {-1, 1, -sx, sx, -sxy, sxy};
	const bool ok[6] = {i > 0, i < sx - 1, j > 0, j < sy - 1, k > 0, k < sz - 1};
	int cnt = 0;
	T s0 = T(0), s1 = T(0), s2 = T(0);
#pragma unroll
	for (int q = 0; q < 2 * D; q++) {
		if (!ok[q]) continue;
		const int n = id + off[q];
		if (!vis0[n]) continue;
		cnt++;
		if (Kind == 0) { s0 += f0[n]; if (NS > 1) s1 += f1[n]; }
		else if (Kind == 1) { s0 += f0[n]; s1 += f1[n]; if (D == 3) s2 += f2[n]; }
	}
	if (cnt > 0) {
		const T c = T(cnt);
		if (Kind == 0) { f0[id] = s0 / c; if (NS > 1) f1[id] = s1 / c; }
		else if (Kind == 1) { f0[id] = s0 / c; f1[id] = s1 / c; if (D == 3) f2[id] = s2 / c; }
		else flag[id] = 1;
		vis1[id] = 1;
	} else {
		if (Kind == 1) {
			const G<D, T> g = cellGrid<D, T>(geom);
			f0[id] = g.pos(0, i); f1[id] = g.pos(1, j); if (D == 3) f2[id] = g.pos(2, k);
		}
		vis1[id] = 0;
	}
}

__global__ void kFlagFinal(int64_t N, uint8_t *flag, const uint8_t *vis0) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id < N && !vis0[id]) flag[id] = 0;
}

template <typename T>
__global__ void kAdvFromOri(int64_t N, const T *ori, uint8_t *adv) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id < N) adv[id] = ori[id] <= T(0) ? 1 : 0;
}

// Liquid faces of extrapolateFieldsToAir (LevelSetLiquid.cpp:1074-1082)
template <int D, typename T>
__global__ void kFaceMask(Geom geom, const T *fr0, const T *fr1, const T *fr2, const T *ori, uint8_t *vis, int64_t F0, int64_t F1, int64_t Ftot) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	const int64_t gid = id;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const T *fr = axis == 0 ? fr0 : (axis == 1 ? fr1 : fr2);
	uint8_t m = 0;
	if (fr[id] < T(1)) {
		const G<D, T> fg = faceGrid<D, T>(geom, axis);
		const G<D, T> cg = cellGrid<D, T>(geom);
		int i, j, k; fg.coord(id, i, j, k);
		const int i0 = i - (axis == 0), j0 = j - (axis == 1), k0 = k - (axis == 2);
		if (cg.valid(i, j, k) && cg.valid(i0, j0, k0))  // always true for interior faces (fraction < 1)
			m = (ori[cg.idx(i0, j0, k0)] <= T(0) || ori[cg.idx(i, j, k)] <= T(0)) ? 1 : 0;
	}
	vis[gid] = m;
}

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kExtrapFacePass(Geom geom, T *u0, T *u1, T *u2, const uint8_t *__restrict__ vis0, uint8_t *vis1, int64_t F0, int64_t F1, int64_t Ftot) {
	const int gid = int(blockIdx.x) * blockDim.x + threadIdx.x;
	if (gid >= int(Ftot)) return;
	if (vis0[gid]) { vis1[gid] = 1; return; }
	int id = gid, axis = 0, base = 0;
	if (id >= int(F0)) { id -= int(F0); axis = 1; base = int(F0); if (id >= int(F1)) { id -= int(F1); axis = 2; base = int(F0 + F1); } }
	const int sx = geom.n[0] + (axis == 0), sy = geom.n[1] + (axis == 1), sz = D == 3 ? geom.n[2] + (axis == 2) : 1;
	T *u = axis == 0 ? u0 : (axis == 1 ? u1 : u2);
	const unsigned r = unsigned(id) / unsigned(sx);
	const int i = id - int(r) * sx;
	const int j = D == 3 ? int(r % unsigned(sy)) : int(r);
	const int k = D == 3 ? int(r / unsigned(sy)) : 0;
	const int sxy = sx * sy;
	const int off[6] = {-1, 1, -sx, sx, -sxy, sxy};
	const bool ok[6] = {i > 0, i < sx - 1, j > 0, j < sy - 1, k > 0, k < sz - 1};
	int cnt = 0; T s = T(0);
#pragma unroll
	for (int q = 0; q < 2 * D; q++) {
		if (!ok[q]) continue;
		const int n = id + off[q];
		if (!vis0[base + n]) continue;
		cnt++; s += u[n];
	}
	if (cnt > 0) { u[id] = s / T(cnt); vis1[gid] = 1; }
	else { u[id] = T(0); vis1[gid] = 0; }
}

template <int D, typename T, int Kind, int NS>
static garm_status cellExtrap(State &s, T *f0, T *f1, T *f2, uint8_t *flag, int passes) {
	uint8_t *v0 = s.vis0, *v1 = s.vis1;
	for (int it = 0; it < passes; it++) {
		kExtrapCellPass<D, T, Kind, NS><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, f0, f1, f2, flag, v0, v1, s.gate); s.launches++;
		uint8_t *t = v0; v0 = v1; v1 = t;
	}
	GARM_CHECK_LAUNCH();
	if (Kind == 2) { kFlagFinal<<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, flag, v0); s.launches++; GARM_CHECK_LAUNCH(); }
	return GARM_OK;
}

static inline int passCount(double r) { int n = 0; while (n < r) n++; return n; }  // `for (iter = 0; iter < maxSteps; ...)`

template <int D, typename T>
garm_status extrapolateToCollider(State &s) {
	kCellMask<T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, kFixedCellDistPos, (const T *)s.cellDist, s.adv, (const T *)s.ori, s.vis0, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	// ori and φ share the fixed set cellDist > 0, so one pass extrapolates both
	return cellExtrap<D, T, 0, 2>(s, (T *)s.ori, (T *)s.phi, nullptr, nullptr, passCount(s.cfg.boundary_extrap_radius));
}

template <int D, typename T>
garm_status extrapolateToAir(State &s) {
	const int R = passCount(s.cfg.air_extrap_radius);
	// ξ from cells with advRegion > 0
	kCellMask<T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, kFixedAdvPos, (const T *)s.cellDist, s.adv, (const T *)s.ori, s.vis0, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	GARM_TRY((cellExtrap<D, T, 1, 1>(s, (T *)s.xi[0], (T *)s.xi[1], (T *)(D == 3 ? s.xi[2] : nullptr), nullptr, R)));
	// advRegion = (ori <= 0), then dilate
	kAdvFromOri<T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, (const T *)s.ori, s.adv); s.launches++;
	kCellMask<T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, kFixedOriNonPos, (const T *)s.cellDist, s.adv, (const T *)s.ori, s.vis0, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	GARM_TRY((cellExtrap<D, T, 2, 1>(s, nullptr, nullptr, nullptr, s.adv, R)));
	// velocity, airExtrapolationRadius + 2 passes
	kFaceMask<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (const T *)s.fraction[0], (const T *)s.fraction[1], (const T *)s.fraction[2],
		(const T *)s.ori, s.fvis0, s.F[0], s.F[1], s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();
	uint8_t *v0 = s.fvis0, *v1 = s.fvis1;
	const int Ru = passCount(s.cfg.air_extrap_radius + 2);
	for (int it = 0; it < Ru; it++) {
		kExtrapFacePass<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (T *)s.u[0], (T *)s.u[1], (T *)s.u[2], v0, v1, s.F[0], s.F[1], s.Ftot); s.launches++;
		uint8_t *t = v0; v0 = v1; v1 = t;
	}
	GARM_CHECK_LAUNCH();
	return GARM_OK;
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

template <int D, typename T>
garm_status maxSpeedAsync(State &s) {
	cudaError_t e = cudaMemsetAsync(s.redU64, 0, sizeof(unsigned long long), s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
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
