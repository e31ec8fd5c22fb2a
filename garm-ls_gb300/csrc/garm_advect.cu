// garm_advect.cu — advectFields (Source/Core/LevelSetLiquid.cpp:718-832), GA branch:
//   1. ∇u per face grid, central 2nd order (Derivatives::computeFirst<2>, Derivatives.h:98-105)
//   2. Hermite mixed derivatives of ξ from Π (HermiteIntrpl ctor, HermiteIntrpl.h:17-30)
//   3. ξ, Π: RK2 traceDrv + Hermite value/gradient, Π' = ∇H(X)·∂X/∂x
//      (Advection.h:71-82, 147-160)
//   4. u: RK2 trace + cubic Lagrange sample (Advection.h:38-43, 137-145; LagrangeIntrpl.h:128-171)
#include "garm_internal.h"

namespace garm {

// ---- 1. velocity gradient: one thread per face over the concatenated face grids
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kVelocityGrad(Geom geom, const T *__restrict__ u0, const T *__restrict__ u1, const T *__restrict__ u2,
                                                        T *g00, T *g01, T *g02, T *g10, T *g11, T *g12, T *g20, T *g21, T *g22,
                                                        int64_t F0, int64_t F1, int64_t Ftot) {
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, T> g = faceGrid<D, T>(geom, axis);
	const T *u = axis == 0 ? u0 : (axis == 1 ? u1 : u2);
	T *out[3];
	if (axis == 0) { out[0] = g00; out[1] = g01; out[2] = g02; }
	else if (axis == 1) { out[0] = g10; out[1] = g11; out[2] = g12; }
	else { out[0] = g20; out[1] = g21; out[2] = g22; }
	int i, j, k;
	g.coord(id, i, j, k);
	const T h = T(0.5) * g.inv;
	out[0][id] = (ldg(u + g.cidx(i + 1, j, k)) - ldg(u + g.cidx(i - 1, j, k))) * h;
	out[1][id] = (ldg(u + g.cidx(i, j + 1, k)) - ldg(u + g.cidx(i, j - 1, k))) * h;
	if (D == 3) out[2][id] = (ldg(u + g.cidx(i, j, k + 1)) - ldg(u + g.cidx(i, j, k - 1))) * h;
}

// ---- 2. Hermite mixed derivatives of a D-component cell field from its gradient planes.
// grad plane (a*D + c) = ∂f_c/∂x_a.  Output plane (m*D + c).
template <int D, typename T>
struct Planes { const T *p[9]; };
template <int D, typename T>
struct OutPlanes { T *p[12]; };

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kMixedVec(Geom geom, Planes<D, T> grad, OutPlanes<D, T> mixed, int ncomp, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T h = T(0.5) * g.inv;
	for (int c = 0; c < ncomp; c++) {
		const T *gy = grad.p[1 * ncomp + c];
		mixed.p[0 * ncomp + c][id] = (ldg(gy + g.cidx(i + 1, j, k)) - ldg(gy + g.cidx(i - 1, j, k))) * h;
		if (D == 3) {
			const T *gz = grad.p[2 * ncomp + c];
			mixed.p[1 * ncomp + c][id] = (ldg(gz + g.cidx(i + 1, j, k)) - ldg(gz + g.cidx(i - 1, j, k))) * h;
			mixed.p[2 * ncomp + c][id] = (ldg(gz + g.cidx(i, j + 1, k)) - ldg(gz + g.cidx(i, j - 1, k))) * h;
			mixed.p[3 * ncomp + c][id] = (ldg(gz + g.cidx(i + 1, j + 1, k)) - ldg(gz + g.cidx(i - 1, j + 1, k)) -
			                              ldg(gz + g.cidx(i + 1, j - 1, k)) + ldg(gz + g.cidx(i - 1, j - 1, k))) * (T(0.25) * g.inv * g.inv);
		}
	}
}

template <int D, typename T>
struct VelView {
	const T *u[3];
	const T *grad[9];  // [axis*3 + b]
	G<D, T> fg[3];
};

// flow(pos) and flow.gradient(pos) of DrvVectorFieldWrapper<SGrid, LinearIntrpl> (VectorField.h:106-138).
// grd[a*D+b] = ∂u_a/∂x_b (row a).
template <int D, typename T, bool WithGrad>
__device__ __forceinline__ void sampleFlow(const VelView<D, T> &v, const T *p, T *vel, T *grd) {
#pragma unroll
	for (int a = 0; a < D; a++) {
		if (WithGrad) {
			const T *planes[D + 1];
			planes[0] = v.u[a];
#pragma unroll
			for (int b = 0; b < D; b++) planes[1 + b] = v.grad[a * 3 + b];
			T out[D + 1];
			lerpN<D, T, D + 1>(planes, v.fg[a], p, out);
			vel[a] = out[0];
#pragma unroll
			for (int b = 0; b < D; b++) grd[a * D + b] = out[1 + b];
		} else {
			vel[a] = lerpNested<D, T>(v.u[a], v.fg[a], p);
		}
	}
}

// ---- 3. GA semi-Lagrangian advection of ξ and Π (one thread per cell)
template <int D, typename T>
struct RefMapIO {
	const T *xi[3];
	const T *Pi[9];      // plane col*D+row
	const T *mixed[12];  // plane m*D+c
	T *xiOut[3];
	T *PiOut[9];
};

// In FP32, three resident blocks per SM (at most 80 registers; 48 bytes spill): the kernel
// waits on its gathers, and 24 warps per SM against 16 took the 128^3 mixed advection from
// 0.745 to 0.656 ms per step.  FP64 keeps the unconstrained form (a cap spills heavily).
template <int D, typename T>
__global__ void __launch_bounds__(kBlock, sizeof(T) == 4 ? 3 : 1) kAdvectRefMap(Geom geom, VelView<D, T> vv, RefMapIO<D, T> io, const double *dtp) {
	const T mdt = T(-*dtp);
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int ci, cj, ck;
	g.coord(id, ci, cj, ck);
	T pos[3] = {g.pos(0, ci), g.pos(1, cj), D == 3 ? g.pos(2, ck) : T(0)};

	// traceDrv<2> (Advection.h:71-82); grd is row-major here: grd[a*D+b] = ∂u_a/∂x_b
	T vel0[D], grd0[D * D], vel1[D], grd1[D * D];
	// The first sample is at the cell centre itself.  In face grid a the centre lies half a
	// cell from the two faces of the cell along a and on a node along the other axes, so the
	// trilinear sample of u_a and of its gradient there is the mean of the cell's two a-faces
	// (LinearIntrpl's weights are exactly 1/2 and 0/1 there; only their rounding is skipped).
#pragma unroll
	for (int a = 0; a < D; a++) {
		const G<D, T> &ga = vv.fg[a];
		const int64_t lo = ga.idx(ci, cj, ck);
		const int64_t hi = ga.idx(ci + (a == 0), cj + (a == 1), ck + (a == 2));
		vel0[a] = (ldg(vv.u[a] + lo) + ldg(vv.u[a] + hi)) * T(0.5);
#pragma unroll
		for (int b = 0; b < D; b++) {
			const T *gp = vv.grad[a * 3 + b];
			grd0[a * D + b] = (ldg(gp + lo) + ldg(gp + hi)) * T(0.5);
		}
	}
	T pos1[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) pos1[a] = pos[a] + vel0[a] * mdt;
	T rot1[D * D];
#pragma unroll
	for (int a = 0; a < D; a++)
#pragma unroll
		for (int b = 0; b < D; b++) rot1[a * D + b] = (a == b ? T(1) : T(0)) + grd0[a * D + b] * mdt;
	sampleFlow<D, T, true>(vv, pos1, vel1, grd1);
	T X[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) X[a] = pos[a] + (vel0[a] + vel1[a]) * mdt / T(2);
	T rot2[D * D];
#pragma unroll
	for (int a = 0; a < D; a++)
#pragma unroll
		for (int b = 0; b < D; b++) {
			T s = grd1[a * D + 0] * rot1[0 * D + b];
#pragma unroll
			for (int k = 1; k < D; k++) s += grd1[a * D + k] * rot1[k * D + b];
			rot2[a * D + b] = (a == b ? T(1) : T(0)) + (grd0[a * D + b] + s) * mdt / T(2);
		}

	// Hermite value and gradient of ξ at X (HermiteIntrpl.h:32-58), tensor-product form.
	int lo[3] = {0, 0, 0};
	T fr[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) { lo[a] = g.lower(a, X[a]); fr[a] = g.frac(a, X[a], lo[a]); }
	T B[3][2][2], Dd[3][2][2];
#pragma unroll
	for (int a = 0; a < D; a++) hermiteBasis<T>(fr[a], g.dx, B[a], Dd[a]);

	// node offsets
	int64_t nid[1 << D];
#pragma unroll
	for (int v = 0; v < (1 << D); v++) {
		const int vi = lo[0] + (v & 1), vj = lo[1] + ((v >> 1) & 1), vk = D == 3 ? lo[2] + (v >> 2) : 0;
		// 64-bit index arithmetic here: with the 32-bit form the compiler overlaps this
		// kernel's 192 gathered loads less and it runs slower
		nid[v] = int64_t(g.cx(vi)) + int64_t(g.s[0]) * (int64_t(g.cy(vj)) + int64_t(g.s[1]) * g.cz(vk));
	}

	T val[D], grad[D * D];  // grad[c*D + a] = ∂ξ_c/∂x_a (before invDx)
	// The interpolant is Σ over vertices v and term orders o of C(v,o)·Π_a B_a[v_a][o_a],
	// and its derivative along a replaces B_a by D_a.  It is contracted one axis at a
	// time, each axis summing over its vertex and its term order together: x for every
	// (y, z) vertex and order (value and d/dx), then y, then z.  Coefficient order o:
	// bit 0 d/dx, bit 1 d/dy, bit 2 d/dz (f, Π col 0, Π col 1, mixed xy, Π col 2,
	// mixed xz, mixed yz, mixed xyz).
#pragma unroll
	for (int c = 0; c < D; c++) {
		auto coefOf = [&](int64_t n, int o) -> T {
			switch (o) {
			case 0: return ldg(io.xi[c] + n);
			case 1: return ldg(io.Pi[0 * D + c] + n);
			case 2: return ldg(io.Pi[1 * D + c] + n);
			case 3: return ldg(io.mixed[0 * D + c] + n);
			case 4: return ldg(io.Pi[2 * D + c] + n);
			case 5: return ldg(io.mixed[1 * D + c] + n);
			case 6: return ldg(io.mixed[2 * D + c] + n);
			default: return ldg(io.mixed[3 * D + c] + n);
			}
		};
		if (D == 2) {
			T X0[2][2], X1[2][2];  // [vy][oy]: x-contracted value and d/dx
#pragma unroll
			for (int vy = 0; vy < 2; vy++) {
				const int64_t n0 = nid[vy << 1 | 0], n1 = nid[vy << 1 | 1];
#pragma unroll
				for (int oy = 0; oy < 2; oy++) {
					const T a0 = coefOf(n0, oy << 1 | 0), a1 = coefOf(n0, oy << 1 | 1);
					const T b0 = coefOf(n1, oy << 1 | 0), b1 = coefOf(n1, oy << 1 | 1);
					X0[vy][oy] = fma(a0, B[0][0][0], fma(a1, B[0][0][1], fma(b0, B[0][1][0], b1 * B[0][1][1])));
					X1[vy][oy] = fma(a0, Dd[0][0][0], fma(a1, Dd[0][0][1], fma(b0, Dd[0][1][0], b1 * Dd[0][1][1])));
				}
			}
			T v = T(0), gx = T(0), gy = T(0);
#pragma unroll
			for (int vy = 0; vy < 2; vy++)
#pragma unroll
				for (int oy = 0; oy < 2; oy++) {
					v = fma(X0[vy][oy], B[1][vy][oy], v);
					gx = fma(X1[vy][oy], B[1][vy][oy], gx);
					gy = fma(X0[vy][oy], Dd[1][vy][oy], gy);
				}
			val[c] = v; grad[c * D + 0] = gx; grad[c * D + 1] = gy;
		} else {
			T Y0[2][2], Yx[2][2], Yy[2][2];  // [vz][oz]: xy-contracted value, d/dx, d/dy
#pragma unroll
			for (int vz = 0; vz < 2; vz++)
#pragma unroll
				for (int oz = 0; oz < 2; oz++) { Y0[vz][oz] = T(0); Yx[vz][oz] = T(0); Yy[vz][oz] = T(0); }
#pragma unroll
			for (int vz = 0; vz < 2; vz++)
#pragma unroll
				for (int vy = 0; vy < 2; vy++) {
					const int64_t n0 = nid[vz << 2 | vy << 1 | 0], n1 = nid[vz << 2 | vy << 1 | 1];
#pragma unroll
					for (int oz = 0; oz < 2; oz++)
#pragma unroll
						for (int oy = 0; oy < 2; oy++) {
							const int o = oz << 2 | oy << 1;
							const T a0 = coefOf(n0, o), a1 = coefOf(n0, o | 1);
							const T b0 = coefOf(n1, o), b1 = coefOf(n1, o | 1);
							const T x0 = fma(a0, B[0][0][0], fma(a1, B[0][0][1], fma(b0, B[0][1][0], b1 * B[0][1][1])));
							const T x1 = fma(a0, Dd[0][0][0], fma(a1, Dd[0][0][1], fma(b0, Dd[0][1][0], b1 * Dd[0][1][1])));
							Y0[vz][oz] = fma(x0, B[1][vy][oy], Y0[vz][oz]);
							Yx[vz][oz] = fma(x1, B[1][vy][oy], Yx[vz][oz]);
							Yy[vz][oz] = fma(x0, Dd[1][vy][oy], Yy[vz][oz]);
						}
				}
			T v = T(0), gx = T(0), gy = T(0), gz = T(0);
#pragma unroll
			for (int vz = 0; vz < 2; vz++)
#pragma unroll
				for (int oz = 0; oz < 2; oz++) {
					v = fma(Y0[vz][oz], B[2][vz][oz], v);
					gx = fma(Yx[vz][oz], B[2][vz][oz], gx);
					gy = fma(Yy[vz][oz], B[2][vz][oz], gy);
					gz = fma(Y0[vz][oz], Dd[2][vz][oz], gz);
				}
			val[c] = v; grad[c * D + 0] = gx; grad[c * D + 1] = gy; grad[c * D + 2] = gz;
		}
	}

	// ξ' = H(X); Π' = (∇H(X) · invDx) · rot2  (Advection.h:158; HermiteIntrpl.h:57)
#pragma unroll
	for (int c = 0; c < D; c++) io.xiOut[c][id] = val[c];
#pragma unroll
	for (int c = 0; c < D; c++)
#pragma unroll
		for (int b = 0; b < D; b++) {
			T s = (grad[c * D + 0] * g.inv) * rot2[0 * D + b];
#pragma unroll
			for (int a = 1; a < D; a++) s += (grad[c * D + a] * g.inv) * rot2[a * D + b];
			io.PiOut[b * D + c][id] = s;  // column b, row c
		}
}

// ---- 4. velocity advection: RK2 trace with trilinear u, cubic Lagrange sample of u_axis
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kAdvectVelocity(Geom geom, VelView<D, T> vv, T *o0, T *o1, T *o2, int64_t F0, int64_t F1, int64_t Ftot, const double *dtp) {
	const T mdt = T(-*dtp);
	int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= Ftot) return;
	int axis = 0;
	if (id >= F0) { id -= F0; axis = 1; if (id >= F1) { id -= F1; axis = 2; } }
	const G<D, T> &g = vv.fg[axis];
	T *out = axis == 0 ? o0 : (axis == 1 ? o1 : o2);
	int i, j, k;
	g.coord(id, i, j, k);
	T pos[3] = {g.pos(0, i), g.pos(1, j), D == 3 ? g.pos(2, k) : T(0)};
	T vel0[D], vel1[D];
	// The flow at the face centre itself (the trace's first sample).  In the face's own grid
	// that is the node value.  In another face grid b the centre lies half a cell from the
	// nodes along the face's axis and along b, and on a node along the third axis, so the
	// trilinear sample there is the mean of four values, at the same clamp-to-edge indices
	// (LinearIntrpl's weights are exactly 1/2 there; only their rounding is skipped).
#pragma unroll
	for (int b = 0; b < D; b++) vel0[b] = faceCentreSample<D, T>(vv.u[b], vv.fg[b], b, axis, i, j, k, id);
	T p1[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) p1[a] = pos[a] + vel0[a] * mdt;
	sampleFlow<D, T, false>(vv, p1, vel1, nullptr);
	T X[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) X[a] = pos[a] + (vel0[a] + vel1[a]) * mdt / T(2);

	// CubicIntrpl (LagrangeIntrpl.h:137-170): lower = floor - 1, frac in [1,2).
	// The reference divides by ±6; multiplying by the rounded 1/6 differs by at most
	// one rounding and keeps two IEEE divisions per axis off the FP64 pipe.
	int lo[3] = {0, 0, 0};
	T w[3][4];
	const T sixth = T(1.0 / 6.0);
#pragma unroll
	for (int a = 0; a < D; a++) {
		lo[a] = g.lower(a, X[a]) - 1;
		const T x = g.frac(a, X[a], lo[a]);
		const T x1 = x - T(1), x2 = x - T(2), x3 = x - T(3);
		w[a][0] = -(x1 * x2 * x3) * sixth;
		w[a][1] = x * x2 * x3 * T(0.5);
		w[a][2] = -(x * x1 * x3) * T(0.5);
		w[a][3] = x * x1 * x2 * sixth;
	}
	const T *u = vv.u[axis];
	int ii[4], jj[4];
#pragma unroll
	for (int t = 0; t < 4; t++) { ii[t] = g.cx(lo[0] + t); jj[t] = g.cy(lo[1] + t); }
	T val = T(0);
	if (D == 2) {
#pragma unroll
		for (int b = 0; b < 4; b++) {
			T sx = T(0);
#pragma unroll
			for (int a = 0; a < 4; a++) sx += ldg(u + g.idx(ii[a], jj[b], 0)) * w[0][a];
			val += sx * w[1][b];
		}
	} else {
#pragma unroll
		for (int c = 0; c < 4; c++) {
			const int kk = g.cz(lo[2] + c);
			T sy = T(0);
#pragma unroll
			for (int b = 0; b < 4; b++) {
				T sx = T(0);
#pragma unroll
				for (int a = 0; a < 4; a++) sx += ldg(u + g.idx(ii[a], jj[b], kk)) * w[0][a];
				sy += sx * w[1][b];
			}
			val += sy * w[2][c];
		}
	}
	out[id] = val;
}

template <int D, typename T>
static VelView<D, T> makeVelView(State &s) {
	VelView<D, T> vv;
	for (int a = 0; a < 3; a++) {
		vv.u[a] = (const T *)s.u[a];
		vv.fg[a] = faceGrid<D, T>(s.geom, a < D ? a : 0);
		for (int b = 0; b < 3; b++) vv.grad[a * 3 + b] = (const T *)s.uGrad[a * 3 + b];
	}
	return vv;
}

template <int D, typename T>
garm_status advectFields(State &s) {
	const int64_t F0 = s.F[0], F1 = s.F[1];
	// u (reads the old velocity for every axis: Advection.h:15-22) needs neither ∇u nor ξ,
	// so it runs beside steps 1-3 on the second stream
	GARM_TRY(forkAux(s, 0));
	{
		const VelView<D, T> vu = makeVelView<D, T>(s);
		kAdvectVelocity<D, T><<<gridFor(s.Ftot), kBlock, 0, s.aux>>>(s.geom, vu, (T *)s.uNew[0], (T *)s.uNew[1], (T *)s.uNew[2], F0, F1, s.Ftot, s.dtDev); s.launches++;
		GARM_CHECK_LAUNCH();
	}
	// 1. ∇u
	kVelocityGrad<D, T><<<gridFor(s.Ftot), kBlock, 0, s.stream>>>(s.geom, (const T *)s.u[0], (const T *)s.u[1], (const T *)s.u[2],
		(T *)s.uGrad[0], (T *)s.uGrad[1], (T *)s.uGrad[2], (T *)s.uGrad[3], (T *)s.uGrad[4], (T *)s.uGrad[5],
		(T *)s.uGrad[6], (T *)s.uGrad[7], (T *)s.uGrad[8], F0, F1, s.Ftot); s.launches++;
	GARM_CHECK_LAUNCH();
	// 2. mixed derivatives of ξ from Π
	Planes<D, T> pg{};
	for (int q = 0; q < D * D; q++) pg.p[q] = (const T *)s.Pi[q];
	OutPlanes<D, T> mo{};
	for (int q = 0; q < 12; q++) mo.p[q] = (T *)s.xiMixed[q];
	kMixedVec<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, pg, mo, D, nullptr); s.launches++;
	GARM_CHECK_LAUNCH();
	// 3. ξ, Π
	VelView<D, T> vv = makeVelView<D, T>(s);
	RefMapIO<D, T> io{};
	for (int c = 0; c < D; c++) { io.xi[c] = (const T *)s.xi[c]; io.xiOut[c] = (T *)s.xiNew[c]; }
	for (int q = 0; q < D * D; q++) { io.Pi[q] = (const T *)s.Pi[q]; io.PiOut[q] = (T *)s.PiNew[q]; }
	for (int q = 0; q < 12; q++) io.mixed[q] = (const T *)s.xiMixed[q];
	kAdvectRefMap<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, vv, io, s.dtDev); s.launches++;
	GARM_CHECK_LAUNCH();
	GARM_TRY(joinAux(s, 0));
	for (int c = 0; c < D; c++) { void *t = s.xi[c]; s.xi[c] = s.xiNew[c]; s.xiNew[c] = t; }
	for (int q = 0; q < D * D; q++) { void *t = s.Pi[q]; s.Pi[q] = s.PiNew[q]; s.PiNew[q] = t; }
	for (int a = 0; a < D; a++) { void *t = s.u[a]; s.u[a] = s.uNew[a]; s.uNew[a] = t; }
	return GARM_OK;
}

template <int D, typename T>
garm_status scalarMixed(State &s, T *const *grad, T *const *mixed) {
	Planes<D, T> pg{};
	for (int a = 0; a < D; a++) pg.p[a] = grad[a];
	OutPlanes<D, T> mo{};
	for (int q = 0; q < (D == 3 ? 4 : 1); q++) mo.p[q] = mixed[q];
	kMixedVec<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, pg, mo, 1, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// Cached mixed derivatives of φ0 (HermiteIntrpl ctor via _refLevelSetView.reset()).
template <int D, typename T>
garm_status resetRefView(State &s) {
	return scalarMixed<D, T>(s, (T *const *)s.refGrad, (T *const *)s.refMixed);
}

#define GARM_INST(D, T) \
	template garm_status advectFields<D, T>(State &); \
	template garm_status resetRefView<D, T>(State &); \
	template garm_status scalarMixed<D, T>(State &, T *const *, T *const *);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
