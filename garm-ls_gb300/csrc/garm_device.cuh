// garm_device.cuh — device-side grid substrate for the GB300 GARM-LS pipeline.
//
// Layout in HBM: every scalar field is one structure-of-arrays plane in the
// reference's x-fastest index order (Source/Core/Grid.h:40-44).  A staggered
// field is D planes, one per face grid; the reference map ξ is D planes and its
// Jacobian Π is D*D planes, plane (col*D+row) = ∂ξ_row/∂x_col, i.e. the column-major
// order of the reference's MatrixDd (Common/Util/Types.h:54).  All reads clamp to
// the edge like GridBasedData::at (Source/Core/GridBasedData.h:47).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace garm {

constexpr int kBlock = 256;

// Geometry of a StaggeredGrid (Source/Core/StaggeredGrid.h:27-36).
struct Geom {
	int dim;
	int n[3];      // cells per axis (resolution, ring included); n[2] == 1 in 2D
	int bw;        // boundary width
	double o[3];   // node-grid origin = center - resolution*dx/2
	double dx, inv_dx;
};

// Rounded arithmetic that the compiler may not contract into FMAs: grid
// positions and lower-corner fractions are computed exactly as the host does.
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }

template <typename T> __device__ __forceinline__ T ldg(const T *p) { return __ldg(p); }

// Programmatic dependent launch (sm_90 and later): a kernel launched with launchPdl may be
// scheduled while the kernel before it on the stream is still finishing.  It calls pdlWait()
// before its first global memory access; that returns once the previous kernel has completed
// and its writes are visible, so every dependency, write-after-read included, still holds.
__device__ __forceinline__ void pdlWait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// A regular sub-grid (node, cell or one face grid): Grid<Dim> (Source/Core/Grid.h:10-61).
template <int D, typename T>
struct G {
	int s[3];
	T org[3];
	T dx, inv;

	__host__ __device__ __forceinline__ int64_t count() const { return int64_t(s[0]) * s[1] * (D == 3 ? s[2] : 1); }
	// Grids hold fewer than 2^31 points (checked at creation), so the linear index of a
	// point of the grid fits 32-bit arithmetic: cheaper than 64-bit multiplies in the
	// gathers that form it for every tap.
	__device__ __forceinline__ int64_t idx(int i, int j, int k) const {
		if (D == 2) return int64_t(i + s[0] * j);
		return int64_t(i + s[0] * (j + s[1] * k));
	}
	__device__ __forceinline__ int cx(int i) const { return min(max(i, 0), s[0] - 1); }
	__device__ __forceinline__ int cy(int j) const { return min(max(j, 0), s[1] - 1); }
	__device__ __forceinline__ int cz(int k) const { return D == 3 ? min(max(k, 0), s[2] - 1) : 0; }
	__device__ __forceinline__ int64_t cidx(int i, int j, int k) const { return idx(cx(i), cy(j), cz(k)); }
	__device__ __forceinline__ bool valid(int i, int j, int k) const {
		return i >= 0 && i < s[0] && j >= 0 && j < s[1] && (D == 2 || (k >= 0 && k < s[2]));
	}
	// Linear index -> coordinates.  Grids hold fewer than 2^31 points (checked at
	// creation), so 32-bit unsigned division is exact and far cheaper than 64-bit.
	__device__ __forceinline__ void coord(int64_t id, int &i, int &j, int &k) const {
		const unsigned u = unsigned(id), sx = unsigned(s[0]);
		const unsigned r = u / sx;
		i = int(u - r * sx);
		if (D == 2) { j = int(r); k = 0; }
		else { const unsigned sy = unsigned(s[1]); const unsigned q = r / sy; j = int(r - q * sy); k = int(q); }
	}
	// position = origin + coord * spacing (Grid.h:37)
	__device__ __forceinline__ T pos(int a, int c) const { return add_rn(org[a], mul_rn(T(c), dx)); }
	// getLinearLower / getLowerFrac (Grid.h:52,55)
	__device__ __forceinline__ int lower(int a, T p) const { return int(floor(mul_rn(sub_rn(p, org[a]), inv))); }
	__device__ __forceinline__ T frac(int a, T p, int lo) const { return mul_rn(sub_rn(sub_rn(p, org[a]), mul_rn(T(lo), dx)), inv); }
};

// Grid factories for the staggered layout (StaggeredGrid.h:31-34, 104-119).
template <int D, typename T>
__host__ __device__ inline G<D, T> cellGrid(const Geom &g) {
	G<D, T> r;
	for (int a = 0; a < 3; a++) { r.s[a] = g.n[a]; r.org[a] = T(g.o[a] + 1.0 * g.dx / 2); }
	if (D == 2) r.s[2] = 1;
	r.dx = T(g.dx); r.inv = T(g.inv_dx);
	return r;
}
template <int D, typename T>
__host__ __device__ inline G<D, T> faceGrid(const Geom &g, int axis) {
	G<D, T> r;
	for (int a = 0; a < 3; a++) { r.s[a] = g.n[a] + (a == axis ? 1 : 0); r.org[a] = T(g.o[a] + (a == axis ? 0.0 : 1.0) * g.dx / 2); }
	if (D == 2) r.s[2] = 1;
	r.dx = T(g.dx); r.inv = T(g.inv_dx);
	return r;
}
template <int D, typename T>
__host__ __device__ inline G<D, T> nodeGrid(const Geom &g) {
	G<D, T> r;
	for (int a = 0; a < 3; a++) { r.s[a] = g.n[a] + 1; r.org[a] = T(g.o[a]); }
	if (D == 2) r.s[2] = 1;
	r.dx = T(g.dx); r.inv = T(g.inv_dx);
	return r;
}

// Trilinear (bilinear) sample of one plane: LinearIntrpl::interpolate
// (Source/Core/LagrangeIntrpl.h:39-76).
template <int D, typename T>
__device__ __forceinline__ T lerp(const T *__restrict__ f, const G<D, T> &g, const T *p) {
	const int li = g.lower(0, p[0]), lj = g.lower(1, p[1]);
	const T fx = g.frac(0, p[0], li), fy = g.frac(1, p[1], lj);
	const int i0 = g.cx(li), i1 = g.cx(li + 1), j0 = g.cy(lj), j1 = g.cy(lj + 1);
	const T wx0 = T(1) - fx, wy0 = T(1) - fy;
	if (D == 2) {
		T v = ldg(f + g.idx(i0, j0, 0)) * (wx0 * wy0);
		v += ldg(f + g.idx(i1, j0, 0)) * (fx * wy0);
		v += ldg(f + g.idx(i0, j1, 0)) * (wx0 * fy);
		v += ldg(f + g.idx(i1, j1, 0)) * (fx * fy);
		return v;
	} else {
		const int lk = g.lower(2, p[2]);
		const T fz = g.frac(2, p[2], lk);
		const int k0 = g.cz(lk), k1 = g.cz(lk + 1);
		const T wz0 = T(1) - fz;
		T v = ldg(f + g.idx(i0, j0, k0)) * (wx0 * wy0 * wz0);
		v += ldg(f + g.idx(i1, j0, k0)) * (fx * wy0 * wz0);
		v += ldg(f + g.idx(i0, j1, k0)) * (wx0 * fy * wz0);
		v += ldg(f + g.idx(i1, j1, k0)) * (fx * fy * wz0);
		v += ldg(f + g.idx(i0, j0, k1)) * (wx0 * wy0 * fz);
		v += ldg(f + g.idx(i1, j0, k1)) * (fx * wy0 * fz);
		v += ldg(f + g.idx(i0, j1, k1)) * (wx0 * fy * fz);
		v += ldg(f + g.idx(i1, j1, k1)) * (fx * fy * fz);
		return v;
	}
}

// `lerp` of a field on face grid b (`gb`) at the centre of face (i, j, k) of face grid
// `axis`.  For b == axis that is the node value.  Otherwise the centre lies half a cell from
// the nodes of grid b along `axis` and along b, and on a node along the third axis, so the
// trilinear sample is the mean of four values at the same clamp-to-edge indices (the
// weights are exactly 1/2; only their rounding is skipped).  b is a compile-time index in
// the callers' unrolled loops.
template <int D, typename T>
__device__ __forceinline__ T faceCentreSample(const T *__restrict__ f, const G<D, T> &gb, int b, int axis, int i, int j, int k, int64_t ownId) {
	if (b == axis) return ldg(f + ownId);
	T s = T(0);
#pragma unroll
	for (int q = 0; q < 4; q++) {
		const int sa = q & 1, sb = q >> 1;  // lower or upper node along `axis`, along b
		const int xi = i - int(axis == 0 && sa == 0) + int(b == 0 && sb == 1);
		const int yj = j - int(axis == 1 && sa == 0) + int(b == 1 && sb == 1);
		const int zk = k - int(axis == 2 && sa == 0) + int(b == 2 && sb == 1);
		s += ldg(f + gb.cidx(xi, yj, zk));
	}
	return s * T(0.25);
}

// The same trilinear (bilinear) sample as `lerp`, evaluated as nested one-dimensional
// interpolations a + f·(b - a), x first: 7 (3) of them, against 8 weight products and
// their sum.  Equal to `lerp` up to rounding.
template <int D, typename T>
__device__ __forceinline__ T lerpNested(const T *__restrict__ f, const G<D, T> &g, const T *p) {
	const int li = g.lower(0, p[0]), lj = g.lower(1, p[1]);
	const T fx = g.frac(0, p[0], li), fy = g.frac(1, p[1], lj);
	const int i0 = g.cx(li), i1 = g.cx(li + 1), j0 = g.cy(lj), j1 = g.cy(lj + 1);
	auto mix = [](T a, T b, T t) { return fma(t, b - a, a); };
	if (D == 2) {
		const T r0 = mix(ldg(f + g.idx(i0, j0, 0)), ldg(f + g.idx(i1, j0, 0)), fx);
		const T r1 = mix(ldg(f + g.idx(i0, j1, 0)), ldg(f + g.idx(i1, j1, 0)), fx);
		return mix(r0, r1, fy);
	} else {
		const int lk = g.lower(2, p[2]);
		const T fz = g.frac(2, p[2], lk);
		const int k0 = g.cz(lk), k1 = g.cz(lk + 1);
		const T r00 = mix(ldg(f + g.idx(i0, j0, k0)), ldg(f + g.idx(i1, j0, k0)), fx);
		const T r10 = mix(ldg(f + g.idx(i0, j1, k0)), ldg(f + g.idx(i1, j1, k0)), fx);
		const T r01 = mix(ldg(f + g.idx(i0, j0, k1)), ldg(f + g.idx(i1, j0, k1)), fx);
		const T r11 = mix(ldg(f + g.idx(i0, j1, k1)), ldg(f + g.idx(i1, j1, k1)), fx);
		return mix(mix(r00, r10, fy), mix(r01, r11, fy), fz);
	}
}

// Trilinear sample of NP planes that share one grid (one set of weights).
template <int D, typename T, int NP>
__device__ __forceinline__ void lerpN(const T *const *f, const G<D, T> &g, const T *p, T *out) {
	const int li = g.lower(0, p[0]), lj = g.lower(1, p[1]);
	const T fx = g.frac(0, p[0], li), fy = g.frac(1, p[1], lj);
	const int i0 = g.cx(li), i1 = g.cx(li + 1), j0 = g.cy(lj), j1 = g.cy(lj + 1);
	const T wx0 = T(1) - fx, wy0 = T(1) - fy;
	if (D == 2) {
		const int64_t c[4] = {g.idx(i0, j0, 0), g.idx(i1, j0, 0), g.idx(i0, j1, 0), g.idx(i1, j1, 0)};
		const T w[4] = {wx0 * wy0, fx * wy0, wx0 * fy, fx * fy};
#pragma unroll
		for (int q = 0; q < NP; q++) {
			T v = T(0);
#pragma unroll
			for (int t = 0; t < 4; t++) v += ldg(f[q] + c[t]) * w[t];
			out[q] = v;
		}
	} else {
		const int lk = g.lower(2, p[2]);
		const T fz = g.frac(2, p[2], lk);
		const int k0 = g.cz(lk), k1 = g.cz(lk + 1);
		const T wz0 = T(1) - fz;
		const int64_t c[8] = {g.idx(i0, j0, k0), g.idx(i1, j0, k0), g.idx(i0, j1, k0), g.idx(i1, j1, k0),
		                      g.idx(i0, j0, k1), g.idx(i1, j0, k1), g.idx(i0, j1, k1), g.idx(i1, j1, k1)};
		const T w[8] = {wx0 * wy0 * wz0, fx * wy0 * wz0, wx0 * fy * wz0, fx * fy * wz0,
		                wx0 * wy0 * fz, fx * wy0 * fz, wx0 * fy * fz, fx * fy * fz};
#pragma unroll
		for (int q = 0; q < NP; q++) {
			T v = T(0);
#pragma unroll
			for (int t = 0; t < 8; t++) v += ldg(f[q] + c[t]) * w[t];
			out[q] = v;
		}
	}
}

// Per-axis cubic Hermite basis and derivative with the dx scaling of the
// derivative terms folded in (HermiteIntrpl.h:89-124, 62-87).
// b[vtx][ord]: vtx = lower/upper node, ord = value/derivative term.
template <typename T>
__device__ __forceinline__ void hermiteBasis(T x, T dx, T b[2][2], T d[2][2]) {
	const T xm1 = x - T(1);
	b[0][0] = (x + x + T(1)) * xm1 * xm1;
	b[1][0] = x * x * (T(3) - x - x);
	b[0][1] = x * xm1 * xm1 * dx;
	b[1][1] = x * x * xm1 * dx;
	d[0][0] = T(6) * x * xm1;
	d[1][0] = T(6) * x * (T(1) - x);
	d[0][1] = (T(3) * x - T(1)) * xm1 * dx;
	d[1][1] = x * (T(3) * x - T(2)) * dx;
}

// Appends this lane's `n` entries (ids[0..n)) to a work list (list/count) with one atomic per
// warp: a warp prefix sum of the lane counts, one atomicAdd by the last lane.
// Every lane of the warp must call it.
__device__ __forceinline__ void warpAppend(int *list, int *count, const int *ids, int n) {
	const unsigned lane = threadIdx.x & 31;
	int incl = n;
#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const int v = __shfl_up_sync(0xffffffffu, incl, o);
		if (lane >= unsigned(o)) incl += v;
	}
	const int total = __shfl_sync(0xffffffffu, incl, 31);
	int base = 0;
	if (lane == 31 && total > 0) base = atomicAdd(count, total);
	base = __shfl_sync(0xffffffffu, base, 31);
	const int start = base + incl - n;
	for (int q = 0; q < n; q++) list[start + q] = ids[q];
}

// 1/x for x in [2^-125, 2^125], by Newton–Raphson iteration for the reciprocal
// (y ← y(1 + e + e²), e = 1 − x·y, the second-order form of y ← y(2 − x·y);
// Muller et al., Handbook of Floating-Point Arithmetic, ch. 4) from the single-
// precision hardware approximation rcp.approx.ftz.f32 (at most 1 ulp of float).
// The FP64 seed is built with integer operations: x's exponent re-biased and the
// top 23 bits of its mantissa make a float within 2^-23 of x, and the float
// result widens back exactly the same way.  The seed is then within 2^-21 of
// 1/x, one refinement leaves e³ < 2^-63, and the result is within 2 ulp of
// the correctly rounded reciprocal.  (The WENO5 weight sums always lie in
// [1, 2^106]: each scaled q lies in [1, 2^27].)
__device__ __forceinline__ double recipPos(double x) {
	const int hi = __double2hiint(x), lo = __double2loint(x);
	const int ex = ((hi >> 20) & 0x7ff) - 1023;
	const unsigned man = (unsigned(hi & 0xfffff) << 3) | (unsigned(lo) >> 29);
	const float xf = __int_as_float(((ex + 127) << 23) | int(man));
	float yf;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(xf));
	const int yb = __float_as_int(yf);
	const int ey = ((yb >> 23) & 0xff) - 127;
	const double y = __hiloint2double(((ey + 1023) << 20) | ((yb & 0x7fffff) >> 3), (yb & 7) << 29);
	const double e = fma(-x, y, 1.0);
	return fma(y, fma(e, e, e), y);
}
__device__ __forceinline__ float recipPos(float x) {
	float y;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
	return fmaf(y, fmaf(-x, y, 1.0f), y);
}

// x normal, positive and inside recipPos's range (false for 0, subnormals, inf, NaN).
__device__ __forceinline__ bool recipRange(double x) {
	const int hi = __double2hiint(x);
	const int ex = ((hi >> 20) & 0x7ff) - 1023;
	return hi > 0 && ex >= -124 && ex <= 124;
}

// Block-wide reductions (warp shuffles, then one warp).
template <typename T>
__device__ __forceinline__ T warpSum(T v) {
#pragma unroll
	for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
	return v;
}
template <typename T>
__device__ __forceinline__ T blockSum(T v, T *sh) {
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	v = warpSum(v);
	if (lane == 0) sh[w] = v;
	__syncthreads();
	const int nw = (blockDim.x + 31) >> 5;
	v = (threadIdx.x < nw) ? sh[threadIdx.x] : T(0);
	if (w == 0) v = warpSum(v);
	__syncthreads();
	return v;  // valid in thread 0
}

}  // namespace garm
