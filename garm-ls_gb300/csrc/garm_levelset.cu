// garm_levelset.cu — level-set stages of LevelSetLiquid::advance:
//   generateCurrentFields   (Source/Core/LevelSetLiquid.cpp:1218-1244)
//   reinitializeLevelSet    (LevelSetLiquid.cpp:1148-1160 → Reinitialization.h:20-80, Derivatives.h:134-159)
//   checkReferenceMap       (LevelSetLiquid.cpp:1246-1283)
//   restart, plain branch   (LevelSetLiquid.cpp:1320-1352)
//   enforceBoundaryLevelSet (LevelSetLiquid.cpp:966-975)
#include "garm_internal.h"
#include "garm_sync.cuh"

#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

namespace garm {

// ---------------------------------------------------------------------------
// generateCurrentFields: φ = H(φ0, ψ0)(ξ); air clamp; solid clamps; tmp; ori
// ---------------------------------------------------------------------------
template <int D, typename T>
struct ComposeIO {
	const T *xi[3];
	const T *ref;
	const T *refGrad[3];
	const T *refMixed[4];
	const uint8_t *adv;
	const T *cellDist;
	T *phi, *tmp, *ori;
	const T *Pi[9];   // Newton configuration: Π (plane col*D+row) ...
	T *lsGrad[3];     // ... and ∇φ = Πᵀ ∇H(ξ) written here (null: not kept)
};

// Scalar Hermite value and gradient at p (HermiteIntrpl::interpolate and
// interpolateGradient, HermiteIntrpl.h:32-58), contracted one axis at a time over
// vertex and term order.  Coefficient order o: bit 0 d/dx, bit 1 d/dy, bit 2 d/dz.
template <int D, typename T>
__device__ __forceinline__ void hermiteValueGrad(const G<D, T> &g, const T *p, const T *f, const T *const *grad, const T *const *mixed,
                                                 T &val, T *gout) {
	int lo[3] = {0, 0, 0};
	T B[3][2][2], Dd[3][2][2];
#pragma unroll
	for (int a = 0; a < D; a++) {
		lo[a] = g.lower(a, p[a]);
		hermiteBasis<T>(g.frac(a, p[a], lo[a]), g.dx, B[a], Dd[a]);
	}
	auto coefOf = [&](int64_t n, int o) -> T {
		switch (o) {
		case 0: return ldg(f + n);
		case 1: return ldg(grad[0] + n);
		case 2: return ldg(grad[1] + n);
		case 3: return ldg(mixed[0] + n);
		case 4: return ldg(grad[2] + n);
		case 5: return ldg(mixed[1] + n);
		case 6: return ldg(mixed[2] + n);
		default: return ldg(mixed[3] + n);
		}
	};
	if (D == 2) {
		T v = T(0), gx = T(0), gy = T(0);
#pragma unroll
		for (int vy = 0; vy < 2; vy++) {
			const int64_t n0 = g.cidx(lo[0], lo[1] + vy, 0), n1 = g.cidx(lo[0] + 1, lo[1] + vy, 0);
#pragma unroll
			for (int oy = 0; oy < 2; oy++) {
				const T a0 = coefOf(n0, oy << 1), a1 = coefOf(n0, oy << 1 | 1), b0 = coefOf(n1, oy << 1), b1 = coefOf(n1, oy << 1 | 1);
				const T x0 = fma(a0, B[0][0][0], fma(a1, B[0][0][1], fma(b0, B[0][1][0], b1 * B[0][1][1])));
				const T x1 = fma(a0, Dd[0][0][0], fma(a1, Dd[0][0][1], fma(b0, Dd[0][1][0], b1 * Dd[0][1][1])));
				v = fma(x0, B[1][vy][oy], v);
				gx = fma(x1, B[1][vy][oy], gx);
				gy = fma(x0, Dd[1][vy][oy], gy);
			}
		}
		val = v; gout[0] = gx * g.inv; gout[1] = gy * g.inv;
	} else {
		T Y0[2][2] = {}, Yx[2][2] = {}, Yy[2][2] = {};
#pragma unroll
		for (int vz = 0; vz < 2; vz++)
#pragma unroll
			for (int vy = 0; vy < 2; vy++) {
				const int64_t n0 = g.cidx(lo[0], lo[1] + vy, lo[2] + vz), n1 = g.cidx(lo[0] + 1, lo[1] + vy, lo[2] + vz);
#pragma unroll
				for (int oz = 0; oz < 2; oz++)
#pragma unroll
					for (int oy = 0; oy < 2; oy++) {
						const int o = oz << 2 | oy << 1;
						const T a0 = coefOf(n0, o), a1 = coefOf(n0, o | 1), b0 = coefOf(n1, o), b1 = coefOf(n1, o | 1);
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
		val = v; gout[0] = gx * g.inv; gout[1] = gy * g.inv; gout[2] = gz * g.inv;
	}
}

// Scalar Hermite value at p (HermiteIntrpl::interpolate, HermiteIntrpl.h:32-41).
template <int D, typename T>
__device__ __forceinline__ T hermiteScalar(const G<D, T> &g, const T *p, const T *f, const T *const *grad, const T *const *mixed) {
	int lo[3] = {0, 0, 0};
	T B[3][2][2], Dd[3][2][2];
#pragma unroll
	for (int a = 0; a < D; a++) {
		lo[a] = g.lower(a, p[a]);
		hermiteBasis<T>(g.frac(a, p[a], lo[a]), g.dx, B[a], Dd[a]);
	}
	T val = T(0);
#pragma unroll
	for (int v = 0; v < (1 << D); v++) {
		const int vb0 = v & 1, vb1 = (v >> 1) & 1, vb2 = (v >> 2) & 1;
		const int64_t n = g.cidx(lo[0] + vb0, lo[1] + vb1, D == 3 ? lo[2] + vb2 : 0);
		if (D == 2) {
			const T c0 = ldg(f + n), c1 = ldg(grad[0] + n), c2 = ldg(grad[1] + n), c3 = ldg(mixed[0] + n);
			const T s0 = c0 * B[0][vb0][0] + c1 * B[0][vb0][1];
			const T s1 = c2 * B[0][vb0][0] + c3 * B[0][vb0][1];
			val += s0 * B[1][vb1][0] + s1 * B[1][vb1][1];
		} else {
			const T c0 = ldg(f + n), c1 = ldg(grad[0] + n), c2 = ldg(grad[1] + n), c3 = ldg(mixed[0] + n);
			const T c4 = ldg(grad[2] + n), c5 = ldg(mixed[1] + n), c6 = ldg(mixed[2] + n), c7 = ldg(mixed[3] + n);
			const T bx0 = B[0][vb0][0], bx1 = B[0][vb0][1];
			const T s00 = c0 * bx0 + c1 * bx1, s10 = c2 * bx0 + c3 * bx1;
			const T s01 = c4 * bx0 + c5 * bx1, s11 = c6 * bx0 + c7 * bx1;
			const T sy0 = s00 * B[1][vb1][0] + s10 * B[1][vb1][1];
			const T sy1 = s01 * B[1][vb1][0] + s11 * B[1][vb1][1];
			val += sy0 * B[2][vb2][0] + sy1 * B[2][vb2][1];
		}
	}
	return val;
}

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kCompose(Geom geom, ComposeIO<D, T> io, T airClamp, T solidTol, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	T p[3] = {io.xi[0][id], io.xi[1][id], D == 3 ? io.xi[2][id] : T(0)};
	T phi;
	if (io.lsGrad[0]) {
		// Newton configuration: _levelSetGrad = Πᵀ ∇H(ξ) (LevelSetLiquid.cpp:1226-1227), before the clamps
		T gr[3] = {T(0), T(0), T(0)};
		hermiteValueGrad<D, T>(g, p, io.ref, io.refGrad, io.refMixed, phi, gr);
#pragma unroll
		for (int a = 0; a < D; a++) {
			T s = T(0);
#pragma unroll
			for (int r = 0; r < D; r++) s = fma(io.Pi[a * D + r][id], gr[r], s);
			io.lsGrad[a][id] = s;
		}
	} else {
		phi = hermiteScalar<D, T>(g, p, io.ref, io.refGrad, io.refMixed);
	}
	if (io.adv[id] == 0 && phi < airClamp) phi = airClamp;
	const T cd = io.cellDist[id];
	if (phi < -cd - solidTol) phi = -cd - solidTol;  // enforceBoundaryLevelSet(φ, 3dx)
	T tmp = phi;
	if (tmp < -cd - T(0)) tmp = -cd - T(0);           // enforceBoundaryLevelSet(tmp, 0)
	io.phi[id] = phi;
	io.tmp[id] = tmp;
	io.ori[id] = phi;
}

template <int D, typename T>
garm_status generateCurrentFields(State &s) {
	ComposeIO<D, T> io{};
	for (int a = 0; a < D; a++) { io.xi[a] = (const T *)s.xi[a]; io.refGrad[a] = (const T *)s.refGrad[a]; }
	for (int m = 0; m < 4; m++) io.refMixed[m] = (const T *)s.refMixed[m];
	io.ref = (const T *)s.ref;
	io.adv = s.adv;
	io.cellDist = (const T *)s.cellDist;
	io.phi = (T *)s.phi; io.tmp = (T *)s.tmp; io.ori = (T *)s.ori;
	if (s.cfg.restart_newton) {
		for (int q = 0; q < D * D; q++) io.Pi[q] = (const T *)s.Pi[q];
		for (int a = 0; a < D; a++) io.lsGrad[a] = (T *)s.lsGrad[a];
	}
	const double airClamp = s.cfg.air_extrap_radius * s.geom.dx;
	kCompose<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, io, T(airClamp), T(3.0 * s.geom.dx), s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// WENO5 reinitialisation (Reinitialization.h:20-80)
// ---------------------------------------------------------------------------
// The scheme (Derivatives.h:134-159) builds both one-sided derivatives of a
// cell from seven values along each axis.  Everything here is arranged around
// one fact: the five differences that give φ⁻ of cell i+1 are the five that
// give φ⁺ of cell i, in reverse order, so the two share their ε, their three
// smoothness indicators and their scaled weights; they differ only in the
// candidate stencils and in which weight goes with which stencil.  A "face
// set" is those five differences around the face between i and i+1.
//
// The arithmetic differs from the reference's order of operations (each
// one-sided derivative is a ratio num/den with the 1/(6 dx) factor applied
// once to the squared sum), so results agree with the FP64 oracle to rounding
// (~1e-13·dx after a full reinitialisation), not bitwise.

// 2^-e for the binary exponent e of x > 0 (x normal, e > -bias): an exact power-of-two
// scale built from the exponent bits, used to keep the WENO weights in range.  With E the
// biased exponent field, the result's field is 2·bias - E: one mask and one subtraction
// in place.
__device__ __forceinline__ double pow2NegExp(double x) {
	return __hiloint2double((2046 << 20) - (__double2hiint(x) & 0x7ff00000), 0);
}
__device__ __forceinline__ float pow2NegExp(float x) {
	return __int_as_float((254 << 23) - (__float_as_int(x) & 0x7f800000));
}
// x·2^-e for the same x: x's significand in [1, 2), equal to x * pow2NegExp(x) (an exact
// product) but formed on the integer pipe by setting the exponent field to the bias.
__device__ __forceinline__ double significandOf(double x) {
	return __hiloint2double((__double2hiint(x) & 0x000fffff) | 0x3ff00000, __double2loint(x));
}
__device__ __forceinline__ float significandOf(float x) {
	return __int_as_float((__float_as_int(x) & 0x007fffff) | 0x3f800000);
}

// max of two non-negative, non-NaN values.  For such values the IEEE bit
// patterns order like the numbers, so an integer max gives exactly fmax and
// keeps the FP64 pipe free.
__device__ __forceinline__ double maxNonNeg(double a, double b) {
	const long long x = __double_as_longlong(a), y = __double_as_longlong(b);
	return __longlong_as_double(x > y ? x : y);
}
__device__ __forceinline__ float maxNonNeg(float a, float b) {
	return __int_as_float(max(__float_as_int(a), __float_as_int(b)));
}
__device__ __forceinline__ bool signBit(double a) { return __double2hiint(a) < 0; }
__device__ __forceinline__ bool signBit(float a) { return __float_as_int(a) < 0; }

// 1/sqrt(x) for x in [2^-120, 2^120]: the FP32 hardware approximation
// rsqrt.approx.ftz.f32 of x (x's mantissa truncated to float; the seed is then within
// about 2^-21 of 1/sqrt(x)) refined by one second-order Newton–Raphson step for the
// inverse square root, y ← y(1 + e/2 + 3e²/8) with e = 1 − x·y² (Muller et al.,
// Handbook of Floating-Point Arithmetic, ch. 4), whose error is about (5/16)e³ < 2^-62:
// within 2 ulp of the correctly rounded value.  Outside the range, or for x = 0, the
// callers use the library functions.
__device__ __forceinline__ bool rsqrtRange(double x) {
	const int ex = ((__double2hiint(x) >> 20) & 0x7ff) - 1023;
	return ex >= -120 && ex <= 120;  // also false for 0, subnormals, inf and NaN
}
// The FP32 hardware approximation of 1/sqrt(x) for x in the range above (x's mantissa
// truncated to float), returned as a double.
__device__ __forceinline__ double rsqrtSeed(double x) {
	const int hi = __double2hiint(x), lo = __double2loint(x);
	const int ex = ((hi >> 20) & 0x7ff) - 1023;
	const unsigned man = (unsigned(hi & 0xfffff) << 3) | (unsigned(lo) >> 29);
	const float xf = __int_as_float(((ex + 127) << 23) | int(man));
	float yf;
	asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yf) : "f"(xf));
	const int yb = __float_as_int(yf);
	const int ey = ((yb >> 23) & 0xff) - 127;
	return __hiloint2double(((ey + 1023) << 20) | ((yb & 0x7fffff) >> 3), (yb & 7) << 29);
}
__device__ __forceinline__ double rsqrtNR(double x) {
	const double y = rsqrtSeed(x);
	const double e = fma(-(x * y), y, 1.0);
	return fma(y, e * fma(e, 0.375, 0.5), y);
}
// sqrt(x) over the same range from the same seed y ≈ 1/sqrt(x): the step runs on
// s = x·y, s ← s(1 + e/2 + 3e²/8) with e = 1 − s·y, so the product with x is not a
// separate instruction; the rounding of x·y enters e and is halved by the step.
__device__ __forceinline__ double sqrtNR(double x) {
	const double y = rsqrtSeed(x);
	const double sq = x * y;
	const double e = fma(-sq, y, 1.0);
	return fma(sq, e * fma(e, 0.375, 0.5), sq);
}
// φ < 0 without an FP64 comparison (-0 counts as not negative, as in the comparison).
__device__ __forceinline__ bool isNegative(double x) {
	const long long b = __double_as_longlong(x);
	return b < 0 && (b << 1) != 0;
}
__device__ __forceinline__ bool isNegative(float x) { return x < 0.f; }

template <typename T> struct WenoConst {
	// ε = 1e-6 max v_k^2 + 1e-99 in FP64 (Derivatives.h:144); FP32 takes 1e-30 as the floor
	// The weights depend only on the ratios of the s_k + ε, so the indicators and ε
	// may carry one common factor.  Every form here uses four times the reference's
	// (cell and column forms: s_k = 13/3 e^2 + f^2; sweep form: Jiang & Peng's
	// 13(x-y)^2 + 3 l^2 divided by 3), which makes each indicator one fma.
	static constexpr T epsScale = T(4e-6);
	static constexpr T floorEps4 = sizeof(T) == 8 ? T(4e-99) : T(4e-30);
};

// One one-sided derivative in ratio form.  num/den · 1/(6 dx) is the derivative.
template <typename T> struct Ratio { T num, den; };

// Scaled squared weights of a face set: with q_k = (s_k+ε)·2^-e (2^e ≤ ε < 2^(e+1),
// an exact scale, so q_k = s_k·2^-e + ε's significand in one rounding) every q_k lies in
// [1, ~7e7], so products of two q_k^2 neither overflow nor underflow in FP32 or FP64;
// α_k = d_k/(s_k+ε)^2 then normalises to the same weights as w_1 = q_2^2 q_3^2,
// w_2 = 6 q_1^2 q_3^2, w_3 = 3 q_1^2 q_2^2 (ten times d_k = .1, .6, .3: each ratio's
// numerator and denominator carry the same factor, and the first weight needs no product).
template <typename T> struct FaceWeights { T a, b, c; };  // a = t2 t3, b = 6 t1 t3, c = t1 t2
template <typename T>
__device__ __forceinline__ FaceWeights<T> faceWeights(T s1, T s2, T s3, T eps) {
	const T sc = pow2NegExp(eps), es = significandOf(eps);
	const T q1 = fma(s1, sc, es), q2 = fma(s2, sc, es), q3 = fma(s3, sc, es);
	const T t1 = q1 * q1, t2 = q2 * q2, t3 = q3 * q3;
	return {t2 * t3, T(6) * (t1 * t3), t1 * t2};
}
// φ⁻ of the cell right of the face: stencils on (E1..E5) with weights (a, b, 3c).
template <typename T>
__device__ __forceinline__ Ratio<T> rightRole(const FaceWeights<T> &w, T P1, T P2, T P3) {
	const T w3 = T(3) * w.c;
	return {fma(w.a, P1, fma(w.b, P2, w3 * P3)), w.a + w.b + w3};
}
// φ⁺ of the cell left of the face: stencils on (E5..E1) with weights (c, b, 3a).
template <typename T>
__device__ __forceinline__ Ratio<T> leftRole(const FaceWeights<T> &w, T R1, T R2, T R3) {
	const T w3 = T(3) * w.a;
	return {fma(w.c, R1, fma(w.b, R2, w3 * R3)), w.c + w.b + w3};
}
// Smoothness indicators of (v1, v2, v3) in the three positions of a face set
// (Derivatives.h:147-149): g = 13/12 (v1-2v2+v3)^2 is common to all three.
// (Derivatives.h:147-149, all four times the reference's: g = 13/3 (v1-2v2+v3)^2 is
// common to the three positions, and the second square enters with weight 1.)
template <typename T> __device__ __forceinline__ T smoothG(T a, T b, T c) { const T e = a - T(2) * b + c; return (T(13.0 / 3.0) * e) * e; }
template <typename T> __device__ __forceinline__ T smoothL(T g, T a, T b, T c) { const T f = a - T(4) * b + T(3) * c; return fma(f, f, g); }
template <typename T> __device__ __forceinline__ T smoothM(T g, T a, T c) { const T f = a - c; return fma(f, f, g); }
template <typename T> __device__ __forceinline__ T smoothR(T g, T a, T b, T c) { const T f = T(3) * a - T(4) * b + c; return fma(f, f, g); }
// Candidate stencils (6× the third-order one-sided values)
template <typename T> __device__ __forceinline__ T stencil1(T a, T b, T c) { return T(2) * a - T(7) * b + T(11) * c; }
template <typename T> __device__ __forceinline__ T stencil2(T a, T b, T c) { return -a + T(5) * b + T(2) * c; }
template <typename T> __device__ __forceinline__ T stencil3(T a, T b, T c) { return T(2) * a + T(5) * b - c; }

// Both one-sided derivatives of one cell from its seven values along an axis
// (weno5 of Derivatives.h:134-159): φ⁻ from the face set D1..D5, φ⁺ from D2..D6.
// The two face sets share two g terms and two candidate stencils.
template <typename T>
__device__ __forceinline__ void wenoCell(const T v[7], Ratio<T> &m, Ratio<T> &p) {
	const T D1 = v[1] - v[0], D2 = v[2] - v[1], D3 = v[3] - v[2], D4 = v[4] - v[3], D5 = v[5] - v[4], D6 = v[6] - v[5];
	const T M = maxNonNeg(maxNonNeg(D2 * D2, D3 * D3), maxNonNeg(D4 * D4, D5 * D5));
	const T epsM = fma(maxNonNeg(M, D1 * D1), WenoConst<T>::epsScale, WenoConst<T>::floorEps4);
	const T epsP = fma(maxNonNeg(M, D6 * D6), WenoConst<T>::epsScale, WenoConst<T>::floorEps4);
	const T g1 = smoothG(D1, D2, D3), g2 = smoothG(D2, D3, D4), g3 = smoothG(D3, D4, D5), g4 = smoothG(D4, D5, D6);
	const FaceWeights<T> wm = faceWeights(smoothL(g1, D1, D2, D3), smoothM(g2, D2, D4), smoothR(g3, D3, D4, D5), epsM);
	const FaceWeights<T> wp = faceWeights(smoothL(g2, D2, D3, D4), smoothM(g3, D3, D5), smoothR(g4, D4, D5, D6), epsP);
	const T P2 = stencil2(D2, D3, D4), P3 = stencil3(D3, D4, D5);
	m = rightRole(wm, stencil1(D1, D2, D3), P2, P3);
	p = leftRole(wp, stencil1(D6, D5, D4), P3, P2);  // stencil2(D5,D4,D3) = P3, stencil3(D4,D3,D2) = P2
}

// Godunov term of one axis (Reinitialization.h:60-70): for φ < 0 keep φ⁻ < 0 and
// φ⁺ > 0, for φ ≥ 0 keep φ⁻ > 0 and φ⁺ < 0; the kept ones enter squared.  The
// sign of a ratio is the sign of its numerator (den > 0), so the choice is made
// on sign bits before any division.
template <typename T>
__device__ __forceinline__ T godunovSq(bool neg, const Ratio<T> &m, const Ratio<T> &p) {
	const T x = signBit(m.num) == neg ? m.num * recipPos(m.den) : T(0);
	const T y = signBit(p.num) != neg ? p.num * recipPos(p.den) : T(0);
	return fma(x, x, y * y);
}

// The pseudo-time update of one sub-stage from the Godunov sum (raw, without the
// (1/(6dx))^2 factor): adv = φ + Δτ·S(φ)·(1 − |∇φ|) with the smoothed sign
// S = φ/sqrt(φ² + (dx|∇φ|)²) (Reinitialization.h:26, 72-75), then the TVD-RK3
// combination of the sub-stage: mode 0 adv, mode 1 (3 base + adv)/4,
// mode 2 (base + 2 adv)/3.
template <typename T, int Mode>
__device__ __forceinline__ T rkUpdate(T f, T rawSum, T k, T dx, T dt, const T *base, int64_t id) {
	T grad, sgn;
	if constexpr (sizeof(T) == 8) {
		grad = (rsqrtRange(rawSum) ? sqrtNR(rawSum) : sqrt(rawSum)) * k;
		const T sp = dx * grad;
		const T q = fma(f, f, sp * sp);
		sgn = f * (rsqrtRange(q) ? rsqrtNR(q) : rsqrt(q));
	} else {
		grad = sqrt(rawSum) * k;
		const T sp = dx * grad;
		sgn = f * rsqrt(fma(f, f, sp * sp));
	}
	const T adv = fma(dt * sgn, T(1) - grad, f);
	if (Mode == 0) return adv;
	if (Mode == 1) return fma(base[id], T(3), adv) * T(0.25);
	return fma(adv, T(2), base[id]) * T(1.0 / 3.0);
}

// ---- Paired FP32 evaluation (FFMA2 / FADD2 / FMUL2 of sm_100 and later): the column form
// evaluates the two in-plane axes of a 3D cell as the two lanes of one float2, so each
// paired instruction does the work of two.  Same formulas as wenoCell / godunovSq; the
// constants are folded into fma forms, so the lanes round differently from the scalar FP32
// code (not from each other).
struct F2 { float2 v; };
__device__ __forceinline__ F2 f2(float a) { return {make_float2(a, a)}; }
__device__ __forceinline__ F2 f2(float a, float b) { return {make_float2(a, b)}; }
__device__ __forceinline__ F2 add2(F2 a, F2 b) { return {__fadd2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 mul2(F2 a, F2 b) { return {__fmul2_rn(a.v, b.v)}; }
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) { return {__ffma2_rn(a.v, b.v, c.v)}; }
__device__ __forceinline__ F2 sub2(F2 a, F2 b) { return fma2(b, f2(-1.f), a); }  // a - b, exact as a subtraction
__device__ __forceinline__ F2 maxNonNeg2(F2 a, F2 b) { return f2(maxNonNeg(a.v.x, b.v.x), maxNonNeg(a.v.y, b.v.y)); }
__device__ __forceinline__ F2 pow2NegExp2(F2 a) { return f2(pow2NegExp(a.v.x), pow2NegExp(a.v.y)); }
// -1/x per lane: the hardware approximation and one Newton–Raphson step y(2 - x y)
// (Muller et al., Handbook of Floating-Point Arithmetic, ch. 4), with the sign folded
// into the step: y·(x y - 2).  Only the square of the quotient is used.
__device__ __forceinline__ F2 negRecip2(F2 x) {
	float a, b;
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(a) : "f"(x.v.x));
	asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(b) : "f"(x.v.y));
	const F2 y = f2(a, b);
	return mul2(y, fma2(x, y, f2(-2.f)));
}
struct Ratio2 { F2 num, den; };
__device__ __forceinline__ F2 smoothG2(F2 a, F2 b, F2 c) { const F2 e = add2(fma2(b, f2(-2.f), a), c); return mul2(mul2(e, f2(float(13.0 / 3.0))), e); }
__device__ __forceinline__ F2 smoothL2(F2 g, F2 a, F2 b, F2 c) { const F2 f = fma2(c, f2(3.f), fma2(b, f2(-4.f), a)); return fma2(f, f, g); }
__device__ __forceinline__ F2 smoothM2(F2 g, F2 a, F2 c) { const F2 f = sub2(a, c); return fma2(f, f, g); }
__device__ __forceinline__ F2 smoothR2(F2 g, F2 a, F2 b, F2 c) { const F2 f = fma2(b, f2(-4.f), fma2(a, f2(3.f), c)); return fma2(f, f, g); }
__device__ __forceinline__ F2 stencil1_2(F2 a, F2 b, F2 c) { return fma2(a, f2(2.f), fma2(b, f2(-7.f), mul2(c, f2(11.f)))); }
__device__ __forceinline__ F2 stencil2_2(F2 a, F2 b, F2 c) { return fma2(a, f2(-1.f), fma2(b, f2(5.f), mul2(c, f2(2.f)))); }
__device__ __forceinline__ F2 stencil3_2(F2 a, F2 b, F2 c) { return fma2(c, f2(-1.f), fma2(b, f2(5.f), mul2(a, f2(2.f)))); }
struct FaceWeights2 { F2 a, b, c; };
__device__ __forceinline__ FaceWeights2 faceWeights2(F2 s1, F2 s2, F2 s3, F2 eps) {
	const F2 sc = pow2NegExp2(eps), es = f2(significandOf(eps.v.x), significandOf(eps.v.y));
	const F2 q1 = fma2(s1, sc, es), q2 = fma2(s2, sc, es), q3 = fma2(s3, sc, es);
	const F2 t1 = mul2(q1, q1), t2 = mul2(q2, q2), t3 = mul2(q3, q3);
	return {mul2(t2, t3), mul2(f2(6.f), mul2(t1, t3)), mul2(t1, t2)};
}
__device__ __forceinline__ Ratio2 rightRole2(const FaceWeights2 &w, F2 P1, F2 P2, F2 P3) {
	const F2 w3 = mul2(f2(3.f), w.c);
	return {fma2(w.a, P1, fma2(w.b, P2, mul2(w3, P3))), add2(add2(w.a, w.b), w3)};
}
__device__ __forceinline__ Ratio2 leftRole2(const FaceWeights2 &w, F2 R1, F2 R2, F2 R3) {
	const F2 w3 = mul2(f2(3.f), w.a);
	return {fma2(w.c, R1, fma2(w.b, R2, mul2(w3, R3))), add2(add2(w.c, w.b), w3)};
}
__device__ __forceinline__ void wenoCell2(const F2 v[7], Ratio2 &m, Ratio2 &p) {
	const F2 D1 = sub2(v[1], v[0]), D2 = sub2(v[2], v[1]), D3 = sub2(v[3], v[2]), D4 = sub2(v[4], v[3]), D5 = sub2(v[5], v[4]), D6 = sub2(v[6], v[5]);
	const F2 M = maxNonNeg2(maxNonNeg2(mul2(D2, D2), mul2(D3, D3)), maxNonNeg2(mul2(D4, D4), mul2(D5, D5)));
	const F2 scale = f2(WenoConst<float>::epsScale), floor4 = f2(WenoConst<float>::floorEps4);
	const F2 epsM = fma2(maxNonNeg2(M, mul2(D1, D1)), scale, floor4);
	const F2 epsP = fma2(maxNonNeg2(M, mul2(D6, D6)), scale, floor4);
	const F2 g1 = smoothG2(D1, D2, D3), g2 = smoothG2(D2, D3, D4), g3 = smoothG2(D3, D4, D5), g4 = smoothG2(D4, D5, D6);
	const FaceWeights2 wm = faceWeights2(smoothL2(g1, D1, D2, D3), smoothM2(g2, D2, D4), smoothR2(g3, D3, D4, D5), epsM);
	const FaceWeights2 wp = faceWeights2(smoothL2(g2, D2, D3, D4), smoothM2(g3, D3, D5), smoothR2(g4, D4, D5, D6), epsP);
	const F2 P2 = stencil2_2(D2, D3, D4), P3 = stencil3_2(D3, D4, D5);
	m = rightRole2(wm, stencil1_2(D1, D2, D3), P2, P3);
	p = leftRole2(wp, stencil1_2(D6, D5, D4), P3, P2);
}
// godunovSq of both lanes, summed.
__device__ __forceinline__ float godunovSq2(bool neg, const Ratio2 &m, const Ratio2 &p) {
	const F2 a = mul2(m.num, negRecip2(m.den)), b = mul2(p.num, negRecip2(p.den));
	const F2 x = f2(signBit(m.num.v.x) == neg ? a.v.x : 0.f, signBit(m.num.v.y) == neg ? a.v.y : 0.f);
	const F2 y = f2(signBit(p.num.v.x) != neg ? b.v.x : 0.f, signBit(p.num.v.y) != neg ? b.v.y : 0.f);
	const F2 s = fma2(x, x, mul2(y, y));
	return s.v.x + s.v.y;
}

// Cell form: one thread per cell, seven clamped loads per axis (clamp-to-edge,
// GridBasedData.h:47).  Used where columns give too little parallelism.
template <int D, typename T, int Mode>
__global__ void __launch_bounds__(kBlock) kReinitCells(G<D, T> g, const T *__restrict__ in, const T *base, T *out, T dt) {
	pdlWait();
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T f = ldg(in + id);
	const int sx = g.s[0], sy = g.s[1], sz = D == 3 ? g.s[2] : 1;
	const int sxy = sx * sy;
	const T *line[3] = {in + (id - i), in + (id - j * sx), in + (id - k * sxy)};
	const int lim[3] = {sx - 1, sy - 1, sz - 1};
	const int pos[3] = {i, j, k};
	const int str[3] = {1, sx, sxy};
	const bool neg = isNegative(f);
	const bool inner = i >= 3 && i + 3 < sx && j >= 3 && j + 3 < sy && (D == 2 || (k >= 3 && k + 3 < sz));
	T sum = T(0);
	constexpr bool paired = D == 3 && sizeof(T) == 4;  // FP32 in 3D: x and y as the two lanes
	if constexpr (paired) {
		F2 u[7];
#pragma unroll
		for (int t = 0; t < 7; t++)
			u[t] = inner ? f2(ldg(in + id + (t - 3)), ldg(in + id + (t - 3) * int64_t(sx)))
			             : f2(ldg(line[0] + min(max(i + t - 3, 0), lim[0])), ldg(line[1] + min(max(j + t - 3, 0), lim[1]) * sx));
		Ratio2 m, p;
		wenoCell2(u, m, p);
		sum = godunovSq2(neg, m, p);
	}
#pragma unroll
	for (int a = paired ? 2 : 0; a < D; a++) {
		T v[7];
		if (inner) {
#pragma unroll
			for (int t = 0; t < 7; t++) v[t] = ldg(in + id + (t - 3) * int64_t(str[a]));
		} else {
#pragma unroll
			for (int t = 0; t < 7; t++) v[t] = ldg(line[a] + min(max(pos[a] + t - 3, 0), lim[a]) * str[a]);
		}
		Ratio<T> m, p;
		wenoCell<T>(v, m, p);
		sum += godunovSq(neg, m, p);
	}
	out[id] = rkUpdate<T, Mode>(f, sum, g.inv * T(1.0 / 6.0), g.dx, dt, base, id);
}

// Column form: each thread owns one point of the plane normal to the last axis
// (z in 3D, y in 2D) and walks `chunk` cells along that axis with the seven
// values in registers.  Along the walk each face set is built once and serves
// φ⁺ of the cell below and φ⁻ of the cell above; the in-plane axes use the cell
// form's clamped loads.  Consecutive threads hold consecutive plane points, so
// every load and store is coalesced.
// In-plane values of the column form read from global memory (clamp-to-edge).
struct GlobalPlanes {
	static constexpr bool kStaged = false;
	__device__ __forceinline__ bool ready(int) { return true; }
	__device__ __forceinline__ void release(int) {}
	__device__ __forceinline__ float at(int, int) const { return 0.f; }
};

// The walk of one column (pidx) over cells [w0, w1) of the last axis.  The plane source
// P provides the in-plane stencil values: from global memory, or (3D FP32) from a tile of
// the plane staged in shared memory, for which ready(w) waits and release(w) frees it.
template <int D, typename T, int Mode, class P>
__device__ __forceinline__ void columnWalk(const G<D, T> &g, const T *__restrict__ in, const T *base, T *out, T dt, int pidx, int w0, int w1, P &src) {
	constexpr int W = D - 1;
	const int sx = g.s[0], sy = D == 3 ? g.s[1] : 1;
	const int plane = sx * sy;
	const int sw = g.s[W];
	const int j = D == 3 ? pidx / sx : 0;
	const int i = pidx - j * sx;
	const bool inner = i >= 3 && i + 3 < sx && (D == 2 || (j >= 3 && j + 3 < sy));
	const T *col = in + pidx;
	const T k6 = g.inv * T(1.0 / 6.0);
	// window v[t] = φ at w - 3 + t (clamped)
	T v[7];
#pragma unroll
	for (int t = 0; t < 7; t++) v[t] = ldg(col + int64_t(min(max(w0 - 3 + t, 0), sw - 1)) * plane);
	// φ⁻ of cell w0 from the face set below it (values w0-3 .. w0+2)
	Ratio<T> mW;
	{
		const T E1 = v[1] - v[0], E2 = v[2] - v[1], E3 = v[3] - v[2], E4 = v[4] - v[3], E5 = v[5] - v[4];
		const T Q = maxNonNeg(maxNonNeg(maxNonNeg(E1 * E1, E2 * E2), maxNonNeg(E3 * E3, E4 * E4)), E5 * E5);
		const T eps = fma(Q, WenoConst<T>::epsScale, WenoConst<T>::floorEps4);
		const FaceWeights<T> fw = faceWeights(smoothL(smoothG(E1, E2, E3), E1, E2, E3), smoothM(smoothG(E2, E3, E4), E2, E4),
		                                      smoothR(smoothG(E3, E4, E5), E3, E4, E5), eps);
		mW = rightRole(fw, stencil1(E1, E2, E3), stencil2(E2, E3, E4), stencil3(E3, E4, E5));
	}
	// differences, their squares and the g terms carried along the walk:
	// E[t] = v[t+1] - v[t] for the face set above the current cell (t = 1..5)
	T E1 = v[2] - v[1], E2 = v[3] - v[2], E3 = v[4] - v[3], E4 = v[5] - v[4], E5 = v[6] - v[5];
	T S1 = E1 * E1, S2 = E2 * E2, S3 = E3 * E3, S4 = E4 * E4, S5 = E5 * E5;
	T gA = smoothG(E1, E2, E3), gB = smoothG(E2, E3, E4);
	const int64_t pstride = plane;
	for (int w = w0; w < w1; w++) {
		if (!src.ready(w)) return;  // a staged plane that never arrived (block-uniform)
		const int64_t id = int64_t(w) * pstride + pidx;
		const T f = v[3];
		const bool neg = isNegative(f);
		// face set above cell w: E1..E5 (values w-2 .. w+3)
		const T gC = smoothG(E3, E4, E5);
		const T Q = maxNonNeg(maxNonNeg(maxNonNeg(S1, S2), maxNonNeg(S3, S4)), S5);
		const FaceWeights<T> fw = faceWeights(smoothL(gA, E1, E2, E3), smoothM(gB, E2, E4), smoothR(gC, E3, E4, E5),
		                                      fma(Q, WenoConst<T>::epsScale, WenoConst<T>::floorEps4));
		const Ratio<T> pW = leftRole(fw, stencil1(E5, E4, E3), stencil2(E4, E3, E2), stencil3(E3, E2, E1));
		const Ratio<T> mNext = rightRole(fw, stencil1(E1, E2, E3), stencil2(E2, E3, E4), stencil3(E3, E4, E5));
		T sum = godunovSq(neg, mW, pW);
		// in-plane axes (threads 3 or more cells from the in-plane edges need no clamping)
		if constexpr (D == 3 && sizeof(T) == 4) {
			// FP32 in 3D: x and y as the two lanes of paired instructions
			F2 u[7];
			if constexpr (P::kStaged) {
#pragma unroll
				for (int t = 0; t < 7; t++) u[t] = f2(src.at(t - 3, 0), src.at(0, t - 3));
			} else if (inner) {
#pragma unroll
				for (int t = 0; t < 7; t++) u[t] = f2(ldg(in + id + (t - 3)), ldg(in + id + (t - 3) * sx));
			} else {
				const T *lx = in + (id - i), *ly = in + (id - int64_t(j) * sx);
#pragma unroll
				for (int t = 0; t < 7; t++) u[t] = f2(ldg(lx + min(max(i + t - 3, 0), sx - 1)), ldg(ly + min(max(j + t - 3, 0), sy - 1) * sx));
			}
			Ratio2 m, p;
			wenoCell2(u, m, p);
			sum += godunovSq2(neg, m, p);
		} else
#pragma unroll
		for (int a = 0; a < D - 1; a++) {
			const int c = a == 0 ? i : j, lim = (a == 0 ? sx : sy) - 1, str = a == 0 ? 1 : sx;
			T u[7];
			if (inner) {
#pragma unroll
				for (int t = 0; t < 7; t++) u[t] = ldg(in + id + (t - 3) * str);
			} else {
				const T *line = in + (id - int64_t(c) * str);
#pragma unroll
				for (int t = 0; t < 7; t++) u[t] = ldg(line + min(max(c + t - 3, 0), lim) * str);
			}
			Ratio<T> m, p;
			wenoCell<T>(u, m, p);
			sum += godunovSq(neg, m, p);
		}
		out[id] = rkUpdate<T, Mode>(f, sum, k6, g.dx, dt, base, id);
		src.release(w);
		// slide the window one cell up
		if (w + 1 < w1) {
#pragma unroll
			for (int t = 0; t < 6; t++) v[t] = v[t + 1];
			v[6] = ldg(col + int64_t(min(w + 4, sw - 1)) * plane);
			E1 = E2; E2 = E3; E3 = E4; E4 = E5; E5 = v[6] - v[5];
			S1 = S2; S2 = S3; S3 = S4; S4 = S5; S5 = E5 * E5;
			gA = gB; gB = gC;
			mW = mNext;
		}
	}
}

template <int D, typename T, int Mode>
__global__ void __launch_bounds__(256) kReinitColumns(G<D, T> g, const T *__restrict__ in, const T *base, T *out, T dt, int chunk) {
	pdlWait();
	const int plane = g.s[0] * (D == 3 ? g.s[1] : 1);
	const int pidx = blockIdx.x * blockDim.x + threadIdx.x;
	if (pidx >= plane) return;
	const int w0 = blockIdx.y * chunk;
	if (w0 >= g.s[D - 1]) return;
	GlobalPlanes src;
	columnWalk<D, T, Mode>(g, in, base, out, dt, pidx, w0, min(w0 + chunk, g.s[D - 1]), src);
}

// ---- Pair form (3D FP32): each thread owns two x-adjacent columns (x even and x + 1) and
// walks them together along z.  Every per-cell quantity of the two cells is the pair of lanes
// of one float2, so the z face sets, the Godunov terms and the update run as paired
// instructions.  Of the three x face sets the two cells need (left of x, between x and x + 1,
// right of x + 1), the outer two are one paired evaluation, the right one with its differences
// in reverse order: a face set evaluated on reversed differences in the φ⁻ role gives the φ⁺
// role of the face set itself (the smoothness indicators and the candidate stencils are
// mirror images).  The shared middle face set is evaluated once and serves φ⁺ of x and φ⁻ of
// x + 1.  The y axis is the paired cell form on the two columns.  Same formulas as the column
// form; the FP32 rounding differs where operations are ordered differently.
constexpr int kPairBlockMax = 256;
__device__ __forceinline__ F2 ldg2(const float *p) { return {__ldg(reinterpret_cast<const float2 *>(p))}; }

// The φ⁻ role of the face set on (E1..E5), both lanes.
__device__ __forceinline__ Ratio2 faceRight2(F2 E1, F2 E2, F2 E3, F2 E4, F2 E5) {
	const F2 Q = maxNonNeg2(maxNonNeg2(maxNonNeg2(mul2(E1, E1), mul2(E2, E2)), maxNonNeg2(mul2(E3, E3), mul2(E4, E4))), mul2(E5, E5));
	const F2 eps = fma2(Q, f2(WenoConst<float>::epsScale), f2(WenoConst<float>::floorEps4));
	const FaceWeights2 fw = faceWeights2(smoothL2(smoothG2(E1, E2, E3), E1, E2, E3), smoothM2(smoothG2(E2, E3, E4), E2, E4),
	                                     smoothR2(smoothG2(E3, E4, E5), E3, E4, E5), eps);
	return rightRole2(fw, stencil1_2(E1, E2, E3), stencil2_2(E2, E3, E4), stencil3_2(E3, E4, E5));
}

// godunovSq of the two cells of a pair (one per lane), each with its own sign of φ.
__device__ __forceinline__ F2 godunovPair(bool negA, bool negB, const Ratio2 &m, const Ratio2 &p) {
	const F2 a = mul2(m.num, negRecip2(m.den)), b = mul2(p.num, negRecip2(p.den));
	const F2 x = f2(signBit(m.num.v.x) == negA ? a.v.x : 0.f, signBit(m.num.v.y) == negB ? a.v.y : 0.f);
	const F2 y = f2(signBit(p.num.v.x) != negA ? b.v.x : 0.f, signBit(p.num.v.y) != negB ? b.v.y : 0.f);
	return fma2(x, x, mul2(y, y));
}

// rkUpdate of the two cells of a pair.
template <int Mode>
__device__ __forceinline__ float2 rkUpdatePair(F2 f, F2 rawSum, float k, float dx, float dt, const float *base, int64_t id) {
	const F2 grad = mul2(f2(sqrtf(rawSum.v.x), sqrtf(rawSum.v.y)), f2(k));
	const F2 sp = mul2(f2(dx), grad);
	const F2 q = fma2(f, f, mul2(sp, sp));
	const F2 sgn = mul2(f, f2(rsqrtf(q.v.x), rsqrtf(q.v.y)));
	const F2 adv = fma2(mul2(f2(dt), sgn), sub2(f2(1.f), grad), f);
	if (Mode == 0) return adv.v;
	const F2 b = ldg2(base + id);
	if (Mode == 1) return mul2(fma2(b, f2(3.f), adv), f2(0.25f)).v;
	return mul2(fma2(adv, f2(2.f), b), f2(1.f / 3.f)).v;
}

template <int Mode>
__global__ void __launch_bounds__(kPairBlockMax) kReinitPairs(G<3, float> g, const float *__restrict__ in, const float *base, float *out, float dt, int chunk) {
	pdlWait();
	const int sx = g.s[0], sy = g.s[1], sz = g.s[2];
	const int hx = sx >> 1;
	const int q = int(blockIdx.x) * int(blockDim.x) + int(threadIdx.x);
	if (q >= hx * sy) return;
	const int w0 = int(blockIdx.y) * chunk;
	if (w0 >= sz) return;
	const int w1 = min(w0 + chunk, sz);
	const int j = q / hx, i = (q - j * hx) * 2;
	const int64_t plane = int64_t(sx) * sy;
	const int pidx = i + j * sx;
	const float *col = in + pidx;
	const bool innerX = i >= 4 && i + 5 < sx, innerY = j >= 3 && j + 3 < sy;
	const float k6 = g.inv * (1.0f / 6.0f);
	const float dx = g.dx;
	// z window of both columns: v[t] = φ at w0 - 3 + t (clamped)
	F2 v[7];
#pragma unroll
	for (int t = 0; t < 7; t++) v[t] = ldg2(col + int64_t(min(max(w0 - 3 + t, 0), sz - 1)) * plane);
	Ratio2 mW = faceRight2(sub2(v[1], v[0]), sub2(v[2], v[1]), sub2(v[3], v[2]), sub2(v[4], v[3]), sub2(v[5], v[4]));
	F2 E1 = sub2(v[2], v[1]), E2 = sub2(v[3], v[2]), E3 = sub2(v[4], v[3]), E4 = sub2(v[5], v[4]), E5 = sub2(v[6], v[5]);
	F2 S1 = mul2(E1, E1), S2 = mul2(E2, E2), S3 = mul2(E3, E3), S4 = mul2(E4, E4), S5 = mul2(E5, E5);
	F2 gA = smoothG2(E1, E2, E3), gB = smoothG2(E2, E3, E4);
	for (int w = w0; w < w1; w++) {
		const int64_t id = int64_t(w) * plane + pidx;
		const F2 f = v[3];
		const bool negA = isNegative(f.v.x), negB = isNegative(f.v.y);
		// z: the face set above the cell pair (values w-2 .. w+3)
		const F2 gC = smoothG2(E3, E4, E5);
		const F2 Q = maxNonNeg2(maxNonNeg2(maxNonNeg2(S1, S2), maxNonNeg2(S3, S4)), S5);
		const FaceWeights2 fw = faceWeights2(smoothL2(gA, E1, E2, E3), smoothM2(gB, E2, E4), smoothR2(gC, E3, E4, E5),
		                                     fma2(Q, f2(WenoConst<float>::epsScale), f2(WenoConst<float>::floorEps4)));
		const Ratio2 pW = leftRole2(fw, stencil1_2(E5, E4, E3), stencil2_2(E4, E3, E2), stencil3_2(E3, E2, E1));
		const Ratio2 mNext = rightRole2(fw, stencil1_2(E1, E2, E3), stencil2_2(E2, E3, E4), stencil3_2(E3, E4, E5));
		F2 sum = godunovPair(negA, negB, mW, pW);
		// x: values x-3 .. x+4 of the row
		{
			float u[8];
			if (innerX) {
#pragma unroll
				for (int t = 0; t < 5; t++) {
					const float2 a = __ldg(reinterpret_cast<const float2 *>(in + id + 2 * t - 4));
					if (t > 0) u[2 * t - 1] = a.x;
					if (2 * t < 8) u[2 * t] = a.y;
				}
			} else {
				const float *row = in + (id - i);
#pragma unroll
				for (int t = 0; t < 8; t++) u[t] = ldg(row + min(max(i + t - 3, 0), sx - 1));
			}
			const float D1 = u[1] - u[0], D2 = u[2] - u[1], D3 = u[3] - u[2], D4 = u[4] - u[3], D5 = u[5] - u[4], D6 = u[6] - u[5], D7 = u[7] - u[6];
			// outer face sets: lane x on (D1..D5) (φ⁻ of x), lane y on (D7..D3) reversed (φ⁺ of x + 1)
			const Ratio2 outer = faceRight2(f2(D1, D7), f2(D2, D6), f2(D3, D5), f2(D4, D4), f2(D5, D3));
			// the middle face set (D2..D6) once; its two roles as the lanes: φ⁺ of x, φ⁻ of x + 1
			const float M = maxNonNeg(maxNonNeg(maxNonNeg(D2 * D2, D3 * D3), maxNonNeg(D4 * D4, D5 * D5)), D6 * D6);
			const FaceWeights<float> wm = faceWeights(smoothL(smoothG(D2, D3, D4), D2, D3, D4), smoothM(smoothG(D3, D4, D5), D3, D5),
			                                          smoothR(smoothG(D4, D5, D6), D4, D5, D6),
			                                          fma(M, WenoConst<float>::epsScale, WenoConst<float>::floorEps4));
			const F2 W1 = f2(wm.c, wm.a), Wb = f2(wm.b), W3 = mul2(f2(3.f), f2(wm.a, wm.c));
			const F2 S1m = stencil1_2(f2(D6, D2), f2(D5, D3), f2(D4, D4));
			const F2 S2m = stencil2_2(f2(D5, D3), f2(D4, D4), f2(D3, D5));
			const F2 S3m = stencil3_2(f2(D4, D4), f2(D3, D5), f2(D2, D6));
			const Ratio2 mid = {fma2(W1, S1m, fma2(Wb, S2m, mul2(W3, S3m))), add2(add2(W1, Wb), W3)};
			const Ratio2 mX = {f2(outer.num.v.x, mid.num.v.y), f2(outer.den.v.x, mid.den.v.y)};
			const Ratio2 pX = {f2(mid.num.v.x, outer.num.v.y), f2(mid.den.v.x, outer.den.v.y)};
			sum = add2(sum, godunovPair(negA, negB, mX, pX));
		}
		// y: the paired cell form on the two columns
		{
			F2 yv[7];
#pragma unroll
			for (int t = 0; t < 7; t++) {
				if (t == 3) { yv[t] = f; continue; }
				yv[t] = innerY ? ldg2(in + id + int64_t(t - 3) * sx) : ldg2(in + (id - int64_t(j) * sx) + int64_t(min(max(j + t - 3, 0), sy - 1)) * sx);
			}
			Ratio2 mY, pY;
			wenoCell2(yv, mY, pY);
			sum = add2(sum, godunovPair(negA, negB, mY, pY));
		}
		*reinterpret_cast<float2 *>(out + id) = rkUpdatePair<Mode>(f, sum, k6, dx, dt, base, id);
		// slide the window one cell up
		if (w + 1 < w1) {
			const F2 zn = ldg2(col + int64_t(min(w + 4, sz - 1)) * plane);
#pragma unroll
			for (int t = 0; t < 6; t++) v[t] = v[t + 1];
			v[6] = zn;
			E1 = E2; E2 = E3; E3 = E4; E4 = E5; E5 = sub2(v[6], v[5]);
			S1 = S2; S2 = S3; S3 = S4; S4 = S5; S5 = mul2(E5, E5);
			gA = gB; gB = gC;
			mW = mNext;
		}
	}
}

// ---- Tiled column form (3D FP32): the in-plane stencils of each z-plane read a tile of
// the plane that the tensor memory accelerator (TMA) stages into shared memory.  A block
// is a 32 x 4 patch of columns; the tile holds x0-4 .. x0+35 (the start rounded down to a
// 16-byte boundary, as TMA requires) and y0-3 .. y0+6 of one plane.  Four planes are in
// flight in a ring of shared-memory slots, each completed on its own mbarrier; one thread
// issues the copies, and a slot is refilled once every thread has passed its plane.
// Blocks whose tile would leave the grid in x or y walk with global loads (the clamped
// edge); so do grids whose rows are not a multiple of 16 bytes.
constexpr int kTileX = 32, kTileY = 4, kTileSlots = 4;
constexpr int kTileRow = kTileX + 8, kTileRows = kTileY + 6;
constexpr int kTileBytes = kTileRow * kTileRows * 4;
constexpr int kTileStride = (kTileBytes + 127) / 128 * 128;
constexpr unsigned long long kTileWaitNs = 1000000000ull;  // a plane not staged within 1 s: error

__device__ __forceinline__ unsigned smemAddr(const void *p) { return unsigned(__cvta_generic_to_shared(p)); }

struct TmaPlanes {
	static constexpr bool kStaged = true;
	const CUtensorMap *map;
	unsigned char *ring;
	unsigned long long *bars;
	int w0, w1, x0, y0, tx, ty;
	int *err;  // the owner's error flag, set when a plane did not arrive in time
	const float *cur = nullptr;

	__device__ void issue(int w) const {
		const int slot = (w - w0) % kTileSlots;
		const unsigned bar = smemAddr(bars + slot), dst = smemAddr(ring + slot * kTileStride);
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(kTileBytes) : "memory");
		asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
		             :: "r"(dst), "l"(reinterpret_cast<unsigned long long>(map)), "r"(x0 - 4), "r"(y0 - 3), "r"(w), "r"(bar) : "memory");
	}
	// Barriers initialised and the first planes requested (every thread calls it).
	__device__ void start() {
		if (threadIdx.x == 0) {
			for (int q = 0; q < kTileSlots; q++)
				asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smemAddr(bars + q)) : "memory");
			asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
		}
		__syncthreads();
		if (threadIdx.x == 0)
			for (int w = w0; w < min(w1, w0 + kTileSlots); w++) issue(w);
	}
	// Bounded wait of the calling thread for plane w's slot; true once the plane is staged.
	__device__ bool waitPlane(int w) const {
		const int slot = (w - w0) % kTileSlots;
		const unsigned bar = smemAddr(bars + slot), parity = unsigned((w - w0) / kTileSlots) & 1u;
		unsigned done = 0;
		unsigned long long start = 0;
		for (unsigned it = 0;; it++) {
			asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
			             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
			if (done) return true;
			if ((it & 255u) == 0) {
				const unsigned long long now = globalNs();
				if (start == 0) start = now;
				else if (now - start > kTileWaitNs) return false;
			}
		}
	}
	// Waits (bounded) until plane w is staged; false in every thread if any gave up.
	// Before a block gives up, thread 0 waits (again bounded) for the other planes still in
	// flight into its ring, so that no issued copy is left writing into the shared memory
	// of a block that has exited.
	__device__ bool ready(int w) {
		const bool done = waitPlane(w);
		if (__syncthreads_or(!done)) {
			if (threadIdx.x == 0) {
				atomicExch(err, 1);
				for (int q = w; q < min(w1, w + kTileSlots); q++) waitPlane(q);
			}
			__syncthreads();
			return false;
		}
		cur = reinterpret_cast<const float *>(ring + ((w - w0) % kTileSlots) * kTileStride);
		return true;
	}
	__device__ __forceinline__ float at(int ox, int oy) const { return cur[(ty + 3 + oy) * kTileRow + tx + 4 + ox]; }
	// Every thread is done with plane w: its slot takes plane w + kTileSlots.
	__device__ void release(int w) {
		__syncthreads();
		if (threadIdx.x == 0 && w + kTileSlots < w1) {
			asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
			issue(w + kTileSlots);
		}
	}
};

template <int Mode>
__global__ void __launch_bounds__(kTileX * kTileY) kReinitColumnsTiled(const __grid_constant__ CUtensorMap map, G<3, float> g, const float *__restrict__ in,
                                                                       const float *base, float *out, float dt, int chunk, int *err) {
	pdlWait();
	__shared__ __align__(128) unsigned char ring[kTileSlots * kTileStride];
	__shared__ __align__(8) unsigned long long bars[kTileSlots];
	const int sx = g.s[0], sy = g.s[1], sz = g.s[2];
	const int tx = int(threadIdx.x) % kTileX, ty = int(threadIdx.x) / kTileX;
	const int x0 = int(blockIdx.x) * kTileX, y0 = int(blockIdx.y) * kTileY;
	const int w0 = int(blockIdx.z) * chunk;
	if (w0 >= sz) return;
	const int w1 = min(w0 + chunk, sz);
	if (!(x0 >= 4 && x0 + kTileX + 4 <= sx && y0 >= 3 && y0 + kTileY + 3 <= sy)) {
		const int i = x0 + tx, j = y0 + ty;
		GlobalPlanes src;
		if (i < sx && j < sy) columnWalk<3, float, Mode>(g, in, base, out, dt, i + j * sx, w0, w1, src);
		return;
	}
	TmaPlanes src{&map, ring, bars, w0, w1, x0, y0, tx, ty, err};
	src.start();
	columnWalk<3, float, Mode>(g, in, base, out, dt, (x0 + tx) + (y0 + ty) * sx, w0, w1, src);
}

// ---- Tiled pair form (3D FP32): the pair form with the in-plane stencils read from a tile of
// each z-plane staged in shared memory by the tensor memory accelerator.  A block is 16 pairs
// (32 cells) by 8 rows of columns; its tile holds x0-4 .. x0+35 (the start on a 16-byte
// boundary, as TMA requires) and y0-3 .. y0+10 of one plane.  The block walks `chunk`
// planes through a ring of four slots.  Each slot has two mbarriers: `full` completes when
// the plane's bytes have landed (one elected thread arms it and issues the copy), `empty`
// when every warp of the block has passed the plane (one arrival per warp).  Thread 0 refills
// the slot of the plane before the one its warp has just finished, so up to three planes are
// staged ahead and no warp waits at a block-wide barrier.  Stencil positions are clamped to
// the grid (clamp-to-edge) before they are looked up in the tile: the clamped position
// always lies inside the tile, so the zero fill TMA writes beyond the grid's edges is never
// read.  Every wait is bounded (kTileWaitNs): past it the block sets the error flag, thread 0
// waits (again bounded) for the copies it issued, and the block returns.
constexpr int kPtX = 16, kPtY = 8, kPtSlots = 4;
constexpr int kPtRow = 2 * kPtX + 8, kPtRows = kPtY + 6;
constexpr int kPtBytes = kPtRow * kPtRows * 4;
constexpr int kPtStride = (kPtBytes + 127) / 128 * 128;

// Bounded wait on one phase of an mbarrier in shared memory; false after kTileWaitNs.
__device__ __forceinline__ bool mbarWait(unsigned bar, unsigned parity) {
	unsigned done = 0;
	unsigned long long start = 0;
	for (unsigned it = 0;; it++) {
		asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
		             : "=r"(done) : "r"(bar), "r"(parity) : "memory");
		if (done) return true;
		if ((it & 255u) == 0) {
			const unsigned long long now = globalNs();
			if (start == 0) start = now;
			else if (now - start > kTileWaitNs) return false;
		}
	}
}

template <int Mode>
__global__ void __launch_bounds__(kPtX * kPtY, 4) kReinitPairsTiled(const __grid_constant__ CUtensorMap map, G<3, float> g, const float *__restrict__ in,
                                                                    const float *base, float *out, float dt, int chunk, int *err) {
	pdlWait();
	__shared__ __align__(128) unsigned char ring[kPtSlots * kPtStride];
	__shared__ __align__(8) unsigned long long fullBar[kPtSlots], emptyBar[kPtSlots];
	const int sx = g.s[0], sy = g.s[1], sz = g.s[2];
	const int tpx = int(threadIdx.x) % kPtX, ty = int(threadIdx.x) / kPtX;
	const int x0 = int(blockIdx.x) * (2 * kPtX), y0 = int(blockIdx.y) * kPtY;
	const int w0 = int(blockIdx.z) * chunk;
	if (w0 >= sz) return;  // the whole block
	const int w1 = min(w0 + chunk, sz);
	const int i = x0 + 2 * tpx, j = y0 + ty;
	const bool active = i < sx && j < sy;  // rows have even length, so i + 1 < sx too
	const int64_t plane = int64_t(sx) * sy;
	const int pidx = min(i, sx - 2) + min(j, sy - 1) * sx;  // inactive threads walk a valid column they do not store
	const float *col = in + pidx;
	const bool innerX = i >= 4 && i + 5 < sx, innerY = j >= 3 && j + 3 < sy;
	const int lxi = i - x0 + 4, lyj = j - y0 + 3;  // the thread's own cell in tile coordinates
	const float k6 = g.inv * (1.0f / 6.0f);
	const float dx = g.dx;
	const unsigned ringBase = smemAddr(ring);
	if (threadIdx.x == 0) {
		for (int q = 0; q < kPtSlots; q++) {
			asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smemAddr(fullBar + q)) : "memory");
			asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smemAddr(emptyBar + q)), "r"(int(blockDim.x) / 32) : "memory");
		}
		asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
		asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
	}
	__syncthreads();
	auto issue = [&](int w) {  // thread 0
		const int slot = (w - w0) % kPtSlots;
		const unsigned bar = smemAddr(fullBar + slot), dst = ringBase + slot * kPtStride;
		asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(bar), "r"(kPtBytes) : "memory");
		asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
		             :: "r"(dst), "l"(reinterpret_cast<unsigned long long>(&map)), "r"(x0 - 4), "r"(y0 - 3), "r"(w), "r"(bar) : "memory");
	};
	int issued = min(w1, w0 + kPtSlots);  // planes [w0, issued) have been requested
	if (threadIdx.x == 0)
		for (int w = w0; w < issued; w++) issue(w);
	// Gives up: flag the error; thread 0 waits (bounded) for the planes it requested and has
	// not seen land, so that no copy is left writing into the shared memory of a block that
	// has returned.
	auto giveUp = [&](int consumed) {
		atomicExch(err, 1);
		if (threadIdx.x == 0)
			for (int w = consumed; w < issued; w++) mbarWait(smemAddr(fullBar + (w - w0) % kPtSlots), unsigned((w - w0) / kPtSlots) & 1u);
	};
	// z window of both columns: v[t] = φ at w0 - 3 + t (clamped)
	F2 v[7];
#pragma unroll
	for (int t = 0; t < 7; t++) v[t] = ldg2(col + int64_t(min(max(w0 - 3 + t, 0), sz - 1)) * plane);
	Ratio2 mW = faceRight2(sub2(v[1], v[0]), sub2(v[2], v[1]), sub2(v[3], v[2]), sub2(v[4], v[3]), sub2(v[5], v[4]));
	F2 E1 = sub2(v[2], v[1]), E2 = sub2(v[3], v[2]), E3 = sub2(v[4], v[3]), E4 = sub2(v[5], v[4]), E5 = sub2(v[6], v[5]);
	F2 S1 = mul2(E1, E1), S2 = mul2(E2, E2), S3 = mul2(E3, E3), S4 = mul2(E4, E4), S5 = mul2(E5, E5);
	F2 gA = smoothG2(E1, E2, E3), gB = smoothG2(E2, E3, E4);
	for (int w = w0; w < w1; w++) {
		const int slot = (w - w0) % kPtSlots;
		// the warp waits together and gives up together (a warp-uniform decision keeps every lane
		// at the __syncwarp below)
		if (!__all_sync(0xffffffffu, mbarWait(smemAddr(fullBar + slot), unsigned((w - w0) / kPtSlots) & 1u))) { giveUp(w); return; }
		const float *tile = reinterpret_cast<const float *>(ring + slot * kPtStride);
		const int64_t id = int64_t(w) * plane + pidx;
		const F2 f = v[3];
		const bool negA = isNegative(f.v.x), negB = isNegative(f.v.y);
		// z: the face set above the cell pair (values w-2 .. w+3)
		const F2 gC = smoothG2(E3, E4, E5);
		const F2 Q = maxNonNeg2(maxNonNeg2(maxNonNeg2(S1, S2), maxNonNeg2(S3, S4)), S5);
		const FaceWeights2 fw = faceWeights2(smoothL2(gA, E1, E2, E3), smoothM2(gB, E2, E4), smoothR2(gC, E3, E4, E5),
		                                     fma2(Q, f2(WenoConst<float>::epsScale), f2(WenoConst<float>::floorEps4)));
		const Ratio2 pW = leftRole2(fw, stencil1_2(E5, E4, E3), stencil2_2(E4, E3, E2), stencil3_2(E3, E2, E1));
		const Ratio2 mNext = rightRole2(fw, stencil1_2(E1, E2, E3), stencil2_2(E2, E3, E4), stencil3_2(E3, E4, E5));
		F2 sum = godunovPair(negA, negB, mW, pW);
		// x: values x-3 .. x+4 of the row, from the tile
		{
			float u[8];
			const float *row = tile + lyj * kPtRow;
			if (innerX) {
#pragma unroll
				for (int t = 0; t < 5; t++) {
					const float2 a = *reinterpret_cast<const float2 *>(row + lxi + 2 * t - 4);
					if (t > 0) u[2 * t - 1] = a.x;
					if (2 * t < 8) u[2 * t] = a.y;
				}
			} else {
#pragma unroll
				for (int t = 0; t < 8; t++) u[t] = row[min(max(i + t - 3, 0), sx - 1) - x0 + 4];
			}
			const float D1 = u[1] - u[0], D2 = u[2] - u[1], D3 = u[3] - u[2], D4 = u[4] - u[3], D5 = u[5] - u[4], D6 = u[6] - u[5], D7 = u[7] - u[6];
			const Ratio2 outer = faceRight2(f2(D1, D7), f2(D2, D6), f2(D3, D5), f2(D4, D4), f2(D5, D3));
			const float M = maxNonNeg(maxNonNeg(maxNonNeg(D2 * D2, D3 * D3), maxNonNeg(D4 * D4, D5 * D5)), D6 * D6);
			const FaceWeights<float> wm = faceWeights(smoothL(smoothG(D2, D3, D4), D2, D3, D4), smoothM(smoothG(D3, D4, D5), D3, D5),
			                                          smoothR(smoothG(D4, D5, D6), D4, D5, D6),
			                                          fma(M, WenoConst<float>::epsScale, WenoConst<float>::floorEps4));
			const F2 W1 = f2(wm.c, wm.a), Wb = f2(wm.b), W3 = mul2(f2(3.f), f2(wm.a, wm.c));
			const F2 S1m = stencil1_2(f2(D6, D2), f2(D5, D3), f2(D4, D4));
			const F2 S2m = stencil2_2(f2(D5, D3), f2(D4, D4), f2(D3, D5));
			const F2 S3m = stencil3_2(f2(D4, D4), f2(D3, D5), f2(D2, D6));
			const Ratio2 mid = {fma2(W1, S1m, fma2(Wb, S2m, mul2(W3, S3m))), add2(add2(W1, Wb), W3)};
			const Ratio2 mX = {f2(outer.num.v.x, mid.num.v.y), f2(outer.den.v.x, mid.den.v.y)};
			const Ratio2 pX = {f2(mid.num.v.x, outer.num.v.y), f2(mid.den.v.x, outer.den.v.y)};
			sum = add2(sum, godunovPair(negA, negB, mX, pX));
		}
		// y: the paired cell form on the two columns, from the tile
		{
			F2 yv[7];
#pragma unroll
			for (int t = 0; t < 7; t++) {
				if (t == 3) { yv[t] = f; continue; }
				const int ly = innerY ? lyj + t - 3 : min(max(j + t - 3, 0), sy - 1) - y0 + 3;
				yv[t] = F2{*reinterpret_cast<const float2 *>(tile + ly * kPtRow + lxi)};
			}
			Ratio2 mY, pY;
			wenoCell2(yv, mY, pY);
			sum = add2(sum, godunovPair(negA, negB, mY, pY));
		}
		const float2 res = rkUpdatePair<Mode>(f, sum, k6, dx, dt, base, id);
		if (active) *reinterpret_cast<float2 *>(out + id) = res;
		// this warp is done with plane w
		__syncwarp();
		if ((threadIdx.x & 31) == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(smemAddr(emptyBar + slot)) : "memory");
		// thread 0 refills the slot of plane w - 1 once every warp has passed it (warp 0 gives up
		// together if that wait runs out)
		if (threadIdx.x < 32 && w - 1 >= w0 && issued < w1) {
			bool ok = true;
			if (threadIdx.x == 0) {
				const int wr = w - 1, rs = (wr - w0) % kPtSlots;
				ok = mbarWait(smemAddr(emptyBar + rs), unsigned((wr - w0) / kPtSlots) & 1u);
				if (ok) {
					asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
					issue(issued);
				}
			}
			if (!__shfl_sync(0xffffffffu, int(ok), 0)) { giveUp(w + 1); return; }
			issued++;
		}
		// slide the window one cell up
		if (w + 1 < w1) {
			const F2 zn = ldg2(col + int64_t(min(w + 4, sz - 1)) * plane);
#pragma unroll
			for (int t = 0; t < 6; t++) v[t] = v[t + 1];
			v[6] = zn;
			E1 = E2; E2 = E3; E3 = E4; E4 = E5; E5 = sub2(v[6], v[5]);
			S1 = S2; S2 = S3; S3 = S4; S4 = S5; S5 = mul2(E5, E5);
			gA = gB; gB = gC;
			mW = mNext;
		}
	}
}

// Tensor maps of the planes the tiled form reads, per (address, shape); encoded on the host
// (cuTensorMapEncodeTiled through the runtime's driver entry point) on first use.
namespace {
struct MapKey {
	const void *p; int sx, sy, sz, box;  // box: 0 the tiled column form's, 1 the tiled pair form's
	bool operator<(const MapKey &o) const {
		if (p != o.p) return p < o.p;
		if (sx != o.sx) return sx < o.sx;
		if (sy != o.sy) return sy < o.sy;
		if (sz != o.sz) return sz < o.sz;
		return box < o.box;
	}
};
std::mutex g_mapMutex;
std::map<MapKey, CUtensorMap> g_maps;
PFN_cuTensorMapEncodeTiled_v12000 encodeTiled() {
	static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
	static bool tried = false;
	if (!tried) {
		tried = true;
		void *f = nullptr;
		cudaDriverEntryPointQueryResult q;
		if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) == cudaSuccess && q == cudaDriverEntryPointSuccess)
			fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
		else cudaGetLastError();
	}
	return fn;
}
}  // namespace

// The tensor map of plane `in` of a 3D FP32 grid with the tile box of the tiled column form
// (boxId 0) or of the tiled pair form (1), or false when it cannot be read that way (rows
// not a multiple of 16 bytes, an unaligned address, no encoder).
static bool tiledMap(const float *in, const G<3, float> &g, CUtensorMap *out, int boxId = 0) {
	const int sx = g.s[0], sy = g.s[1], sz = g.s[2];
	if (sx % 4 != 0 || (reinterpret_cast<uintptr_t>(in) & 15) != 0) return false;
	std::lock_guard<std::mutex> lock(g_mapMutex);
	const MapKey key{in, sx, sy, sz, boxId};
	auto it = g_maps.find(key);
	if (it != g_maps.end()) { *out = it->second; return true; }
	PFN_cuTensorMapEncodeTiled_v12000 enc = encodeTiled();
	if (!enc) return false;
	CUtensorMap m;
	const cuuint64_t dims[3] = {cuuint64_t(sx), cuuint64_t(sy), cuuint64_t(sz)};
	const cuuint64_t strides[2] = {cuuint64_t(sx) * 4, cuuint64_t(sx) * cuuint64_t(sy) * 4};
	const cuuint32_t box[3] = {cuuint32_t(boxId ? kPtRow : kTileRow), cuuint32_t(boxId ? kPtRows : kTileRows), 1};
	const cuuint32_t elem[3] = {1, 1, 1};
	if (enc(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(in), dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
	        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
		return false;
	g_maps[key] = m;
	*out = m;
	return true;
}

// The error flag of the tiled form (a staged plane that did not arrive in time) that the
// launches on `st` write to `err`; synchronises.  The flag stays set: the level set of a
// reinitialisation that gave up is not usable.
garm_status tiledReinitStatus(cudaStream_t st, const int *err) {
	int e = 0;
	if (cudaMemcpyAsync(&e, err, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess) return GARM_CUDA_ERROR;
	if (cudaStreamSynchronize(st) != cudaSuccess) return GARM_CUDA_ERROR;
	return e ? GARM_TIMEOUT : GARM_OK;
}

// Sweep form: three passes per sub-stage, one per axis (x, then y, then z).
// Each thread owns a line along the pass's axis and walks `chunk` cells of it;
// every face set of the line is built once and serves φ⁺ of the cell below it
// and φ⁻ of the cell above it.  The faces use the arrangement of Jiang & Peng
// (2000, "Weighted ENO schemes for Hamilton-Jacobi equations"), an exact
// rewrite of the same weights: a central part 12C(i) = 7(D_i + D_{i+1}) -
// (D_{i-1} + D_{i+2}) shared by both one-sided derivatives of cell i, and a
// correction in T1 = a-2b+c and T2 = b-2c+d, built from the face's second
// differences a..d, whose smoothness indicators are
// 13(x-y)^2 + 3(..)^2 = 12 times the reference's (computed here divided by 3,
// 13/3 (x-y)^2 + (..)^2, with ε scaled alike: see WenoConst):
//   12 φ⁻(i+1) = 12C(i+1) + T2 - (.4 t2t3 T1 + .6 t1t2 T2) / (.1 t2t3 + .6 t1t3 + .3 t1t2)
//   12 φ⁺(i)   = 12C(i)   - T1 + (.4 t1t2 T2 + .6 t2t3 T1) / (.1 t1t2 + .6 t1t3 + .3 t2t3)
// The kernel carries 6φ: with s = D_i + D_{i+1} (cell i = f+1) the bases are
// 6C + T2/2 = 3s - (c-b) and 6C - T2/2 = 3s - (d-c), one fma each, and each
// ratio is halved, then scaled by 5/3 above and below: with U = t2t3 T1 and
// V = t1t2 T2 the numerators are 2/3 U + V and U + 2/3 V over
// 1/3 t2t3 + 2 t1t3 + t1t2 and t2t3 + 2 t1t3 + 1/3 t1t2 (two fma each).  T2 is the
// difference of the third differences c-b and d-c, and g13(c, d) squares the latter.
// Differences, squares, g terms, third differences and central parts slide
// with the walk, so each face set is built once per pass, at about 44
// arithmetic instructions.  The Godunov sum of the first passes goes to `out` (x pass:
// stored, y pass: added); the last pass adds its own and applies the update.
// 13/3 (x-y)^2: the indicators here are 13(x-y)^2 + 3 l^2 divided by 3 (with ε
// alike), so the second square enters with weight 1 (one fma per indicator).
template <typename T> __device__ __forceinline__ T g13(T x, T y) { const T d = x - y; return (T(13.0 / 3.0) * d) * d; }

template <int D, typename T, int A, int Mode>
__global__ void __launch_bounds__(256) kWenoSweep(G<D, T> g, const T *__restrict__ in, const T *base, T *out, T dt, int chunk) {
	pdlWait();
	constexpr int Stage = A == 0 ? 0 : (A == D - 1 ? 2 : 1);
	const int sx = g.s[0], sy = g.s[1], sz = D == 3 ? g.s[2] : 1;
	const int len = g.s[A];
	const int nLines = A == 0 ? sy * sz : (A == 1 ? sx * sz : sx * sy);
	const int L = blockIdx.x * blockDim.x + threadIdx.x;
	if (L >= nLines) return;
	const int w0 = blockIdx.y * chunk;
	if (w0 >= len) return;
	const int w1 = min(w0 + chunk, len);
	int64_t lb, st;
	if (A == 0) { lb = int64_t(L) * sx; st = 1; }
	else if (A == 1) { const int z = L / sx; lb = int64_t(z) * sx * sy + (L - z * sx); st = sx; }
	else { lb = L; st = int64_t(sx) * sy; }
	const T *line = in + lb;
	const int last = len - 1;
	auto ld = [&](int w) { return ldg(line + int64_t(min(max(w, 0), last)) * st); };
	const T epsFloor = WenoConst<T>::floorEps4;  // 12/3 = 4 x the reference's ε
	// state before the face f0 = w0 - 1 (between cells w0-1 and w0): φ_{f0-2 .. f0+2}
	const int f0 = w0 - 1;
	const T p0 = ld(f0 - 2), p1 = ld(f0 - 1);
	T phiF = ld(f0), phiF1 = ld(f0 + 1), phiF2 = ld(f0 + 2);
	const T E1 = p1 - p0, E2 = phiF - p1;                                    // D_{f-1}, D_f
	T E3 = phiF1 - phiF, E4 = phiF2 - phiF1;                                  // D_{f+1}, D_{f+2}
	T Q1 = E1 * E1, Q2 = E2 * E2, Q3 = E3 * E3, Q4 = E4 * E4;
	T a = E2 - E1, b = E3 - E2, c = E4 - E3;                                // Δ_f .. Δ_{f+2}
	T gab = g13(a, b), gbc = g13(b, c);
	T e2 = c - b;                                                             // third difference
	T T1 = e2 - (b - a);
	T dpBase = T(0), dmCarry = T(0);
	const T k = g.inv * T(1.0 / 6.0);
	for (int f = f0; f < w1; f++) {
		const T pn = ld(f + 3);
		const T E5 = pn - phiF2, Q5 = E5 * E5;
		const T d = E5 - E4;
		const T e3 = d - c;
		const T T2 = e3 - e2;                                                 // b - 2c + d
		const T gcd = (T(13.0 / 3.0) * e3) * e3;                              // g13(c, d)
		const T l0 = fma(T(-3), b, a), l1 = b + c, l2 = fma(T(3), c, -d);
		const T is0 = fma(l0, l0, gab), is1 = fma(l1, l1, gbc), is2 = fma(l2, l2, gcd);
		const T Qm = maxNonNeg(maxNonNeg(maxNonNeg(Q1, Q2), maxNonNeg(Q3, Q4)), Q5);
		const T eps = fma(Qm, WenoConst<T>::epsScale, epsFloor);
		const T sc = pow2NegExp(eps), es = significandOf(eps);                  // es = eps·sc
		const T q1 = fma(is0, sc, es), q2 = fma(is1, sc, es), q3 = fma(is2, sc, es);
		const T t1 = q1 * q1, t2 = q2 * q2, t3 = q3 * q3;
		const T Aw = t2 * t3, T13 = t1 * t3, Cw = t1 * t2;
		const T U = Aw * T1, V = Cw * T2;
		const T s = E3 + E4;
		const T denR = fma(T(1.0 / 3.0), Aw, fma(T(2), T13, Cw));
		const T dmNext = fma(-fma(T(2.0 / 3.0), U, V), recipPos(denR), fma(T(3), s, -e2));   // 6 φ⁻(f+1)
		if (f >= w0) {
			const T denL = fma(T(1.0 / 3.0), Cw, fma(T(2), T13, Aw));
			const T dpF = fma(fma(T(2.0 / 3.0), V, U), recipPos(denL), dpBase);             // 6 φ⁺(f)
			const bool neg = isNegative(phiF);
			const T x = signBit(dmCarry) == neg ? dmCarry : T(0);
			const T y = signBit(dpF) != neg ? dpF : T(0);
			const int64_t id = lb + int64_t(f) * st;
			if (Stage == 0) out[id] = fma(x, x, y * y);
			else if (Stage == 1) out[id] = fma(x, x, fma(y, y, out[id]));
			else out[id] = rkUpdate<T, Mode>(phiF, fma(x, x, fma(y, y, out[id])), k, g.dx, dt, base, id);
		}
		dmCarry = dmNext; dpBase = fma(T(3), s, -e3);                           // 6 C(f+1) - T2 / 2
		E3 = E4; E4 = E5;
		Q1 = Q2; Q2 = Q3; Q3 = Q4; Q4 = Q5;
		a = b; b = c; c = d;
		gab = gbc; gbc = gcd;
		e2 = e3; T1 = T2;
		phiF = phiF1; phiF1 = phiF2; phiF2 = pn;
	}
}

// Launch plan of the reinitialisation sub-stages for one grid shape: the cell
// form, the column form or the sweep form, with `block` threads and `chunk`
// cells per thread.  Chosen by timing (reinitPlanFor) and cached per device
// and shape.
enum ReinitForm { kFormCells = GARM_REINIT_CELLS, kFormColumns = GARM_REINIT_COLUMNS, kFormSweeps = GARM_REINIT_SWEEPS, kFormTiled = GARM_REINIT_TILED,
                  kFormPairs = GARM_REINIT_PAIRS, kFormPairsTiled = GARM_REINIT_PAIRS_TILED };

// The pair form reads and writes float2: rows of even length and 8-byte aligned planes.
static bool pairsApply(const G<3, float> &g, const void *in, const void *base, const void *out) {
	const auto a8 = [](const void *p) { return (reinterpret_cast<uintptr_t>(p) & 7) == 0; };
	return g.s[0] % 2 == 0 && a8(in) && a8(out) && (!base || a8(base));
}
struct ReinitPlan { int form = kFormColumns, block = 128, chunk = 8; float ms = 0; };

template <int D, typename T, int A, int Mode>
static void launchSweep(const ReinitPlan &pl, cudaStream_t st, const G<D, T> &g, const T *in, const T *base, T *out, T dt) {
	const int sx = g.s[0], sy = g.s[1], sz = D == 3 ? g.s[2] : 1;
	const int nLines = A == 0 ? sy * sz : (A == 1 ? sx * sz : sx * sy);
	const dim3 grid((nLines + pl.block - 1) / pl.block, (g.s[A] + pl.chunk - 1) / pl.chunk);
	launchPdl(kWenoSweep<D, T, A, Mode>, grid, dim3(pl.block), st, g, in, base, out, dt, pl.chunk);
}

// One sub-stage; returns the number of kernels launched.
template <int D, typename T, int Mode>
static int launchReinit(const ReinitPlan &pl, cudaStream_t st, const G<D, T> &g, const T *in, const T *base, T *out, T dt, int *err) {
	if (pl.form == kFormCells) {
		launchPdl(kReinitCells<D, T, Mode>, dim3(gridFor(g.count())), dim3(kBlock), st, g, in, base, out, dt);
		return 1;
	}
	if (pl.form == kFormSweeps) {
		launchSweep<D, T, 0, Mode>(pl, st, g, in, base, out, dt);
		launchSweep<D, T, 1, Mode>(pl, st, g, in, base, out, dt);
		if (D == 3) launchSweep<D, T, D == 3 ? 2 : 1, Mode>(pl, st, g, in, base, out, dt);
		return D;
	}
	if constexpr (D == 3 && sizeof(T) == 4) {
		if (pl.form == kFormPairs && pairsApply(g, in, base, out)) {
			const int pairs = (g.s[0] / 2) * g.s[1];
			const dim3 grid((pairs + pl.block - 1) / pl.block, (g.s[2] + pl.chunk - 1) / pl.chunk);
			launchPdl(kReinitPairs<Mode>, grid, dim3(pl.block), st, g, (const float *)in, (const float *)base, (float *)out, float(dt), pl.chunk);
			return 1;
		}
		CUtensorMap map;
		if (pl.form == kFormPairsTiled && pairsApply(g, in, base, out) && tiledMap((const float *)in, g, &map, 1)) {
			const dim3 grid((g.s[0] + 2 * kPtX - 1) / (2 * kPtX), (g.s[1] + kPtY - 1) / kPtY, (g.s[2] + pl.chunk - 1) / pl.chunk);
			launchPdl(kReinitPairsTiled<Mode>, grid, dim3(kPtX * kPtY), st, map, g, (const float *)in, (const float *)base, (float *)out, float(dt), pl.chunk, err);
			return 1;
		}
		if (pl.form == kFormPairsTiled && pairsApply(g, in, base, out)) {  // rows not a multiple of 16 bytes: the pair form
			const int pairs = (g.s[0] / 2) * g.s[1];
			const dim3 grid((pairs + 128 - 1) / 128, (g.s[2] + pl.chunk - 1) / pl.chunk);
			launchPdl(kReinitPairs<Mode>, grid, dim3(128), st, g, (const float *)in, (const float *)base, (float *)out, float(dt), pl.chunk);
			return 1;
		}
		if (pl.form == kFormTiled && tiledMap((const float *)in, g, &map)) {
			const dim3 grid((g.s[0] + kTileX - 1) / kTileX, (g.s[1] + kTileY - 1) / kTileY, (g.s[2] + pl.chunk - 1) / pl.chunk);
			launchPdl(kReinitColumnsTiled<Mode>, grid, dim3(kTileX * kTileY), st, map, g, (const float *)in, (const float *)base, (float *)out, float(dt), pl.chunk, err);
			return 1;
		}
	}
	// the column form (also the tiled and pair forms where they do not apply)
	const int block = pl.form == kFormTiled ? kTileX * kTileY : pl.form == kFormPairsTiled ? kPtX * kPtY : pl.block;
	const int plane = g.s[0] * (D == 3 ? g.s[1] : 1);
	const int sw = g.s[D - 1];
	const dim3 grid((plane + block - 1) / block, (sw + pl.chunk - 1) / pl.chunk);
	launchPdl(kReinitColumns<D, T, Mode>, grid, dim3(block), st, g, in, base, out, dt, pl.chunk);
	return 1;
}

namespace {
struct PlanKey {
	int dev, dim, esz, s0, s1, s2;
	bool operator<(const PlanKey &o) const {
		const int a[6] = {dev, dim, esz, s0, s1, s2}, b[6] = {o.dev, o.dim, o.esz, o.s0, o.s1, o.s2};
		for (int q = 0; q < 6; q++) if (a[q] != b[q]) return a[q] < b[q];
		return false;
	}
};
std::mutex g_planMutex;
std::map<PlanKey, ReinitPlan> g_plans;
}  // namespace

// The launch plan for this shape.  The first time a shape is seen on a device
// (outside stream capture) every candidate runs sub-stage 0 (in → out only, so
// the field is untouched) once to warm up and three times timed on the caller's
// stream; the candidate with the smallest time is kept.  The tuning synchronises
// that stream once per candidate.  Under capture, when a timing call fails, or
// when the caller asks for no tuning, the plan is the default column form and
// nothing is cached.
template <int D, typename T>
static ReinitPlan reinitPlanFor(cudaStream_t st, const G<D, T> &g, const T *phi, T *scratch, T dt, int *err, bool tune = true) {
	int dev = 0;
	cudaGetDevice(&dev);
	const PlanKey key{dev, D, int(sizeof(T)), g.s[0], g.s[1], D == 3 ? g.s[2] : 1};
	{
		std::lock_guard<std::mutex> lock(g_planMutex);
		auto it = g_plans.find(key);
		if (it != g_plans.end()) return it->second;
	}
	ReinitPlan best;
	if (!tune) return best;
	cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
	if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) { cudaGetLastError(); return best; }
	std::vector<ReinitPlan> cand;
	cand.push_back({kFormCells, kBlock, 0});
	// walks of the column form: fixed lengths, plus ones that split the walked axis into 4-16
	// equal pieces, so that some block count fits the resident waves well
	std::vector<int> colWalks = {4, 8, 16, 32};
	for (int pieces : {4, 6, 8, 12, 16}) colWalks.push_back((g.s[D - 1] + pieces - 1) / pieces);
	std::sort(colWalks.begin(), colWalks.end());
	colWalks.erase(std::unique(colWalks.begin(), colWalks.end()), colWalks.end());
	for (int b : {64, 128, 256})
		for (int c : colWalks) cand.push_back({kFormColumns, b, c});
	if (D == 3 && sizeof(T) == 4) {
		for (int c : {4, 8, 16, 32}) cand.push_back({kFormTiled, kTileX * kTileY, c});
		if (g.s[0] % 2 == 0) {
			for (int b : {64, 128, 256})
				for (int c : colWalks) cand.push_back({kFormPairs, b, c});
			if (g.s[0] % 4 == 0)
				for (int c : colWalks) cand.push_back({kFormPairsTiled, kPtX * kPtY, c});
		}
	}
	// sweeps: walks that split the longest axis into 2-8 equal pieces, plus short fixed ones
	int longest = 0;
	for (int a = 0; a < D; a++) longest = std::max(longest, g.s[a]);
	std::vector<int> walks = {8, 16};
	for (int pieces : {2, 3, 4, 5, 6, 8}) walks.push_back((longest + pieces - 1) / pieces);
	std::sort(walks.begin(), walks.end());
	walks.erase(std::unique(walks.begin(), walks.end()), walks.end());
	for (int b : {32, 64, 128})
		for (int c : walks) cand.push_back({kFormSweeps, b, c});
	cudaEvent_t e0, e1;
	if (cudaEventCreate(&e0) != cudaSuccess) { cudaGetLastError(); return best; }
	if (cudaEventCreate(&e1) != cudaSuccess) { cudaEventDestroy(e0); cudaGetLastError(); return best; }
	bool ok = true;
	float bestMs = 1e30f;
	for (ReinitPlan &c : cand) {
		launchReinit<D, T, 0>(c, st, g, phi, nullptr, scratch, dt, err);  // warm
		float shortest = 1e30f;
		for (int rep = 0; rep < 3 && ok; rep++) {
			cudaEventRecord(e0, st);
			launchReinit<D, T, 0>(c, st, g, phi, nullptr, scratch, dt, err);
			cudaEventRecord(e1, st);
			if (cudaEventSynchronize(e1) != cudaSuccess) { ok = false; break; }
			float ms = 0;
			cudaEventElapsedTime(&ms, e0, e1);
			shortest = std::min(shortest, ms);
		}
		if (!ok) break;
		c.ms = shortest;
		if (shortest < bestMs) { bestMs = shortest; best = c; }
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	if (!ok || cudaGetLastError() != cudaSuccess) return ReinitPlan{};
	std::lock_guard<std::mutex> lock(g_planMutex);
	g_plans[key] = best;
	return best;
}

// Pin (or, with block 0, forget) the plan of one shape on the current device.
garm_status pinReinitPlan(int dim, int esz, const int *size, int form, int block, int chunk) {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return GARM_CUDA_ERROR; }
	const PlanKey key{dev, dim, esz, size[0], size[1], dim == 3 ? size[2] : 1};
	std::lock_guard<std::mutex> lock(g_planMutex);
	if (block == 0) { g_plans.erase(key); return GARM_OK; }
	ReinitPlan pl;
	pl.form = form;
	pl.block = form == kFormCells ? kBlock : form == kFormTiled ? kTileX * kTileY : form == kFormPairsTiled ? kPtX * kPtY : block;
	pl.chunk = form == kFormCells ? 0 : chunk;
	g_plans[key] = pl;
	return GARM_OK;
}

// Reinitialisation::solve<5> with TVD-RK3 (Reinitialization.h:50-80).  The three
// planes rotate roles every iteration (u0 → X → Y → X holds u0's successor), so
// no sub-stage writes a plane it reads; after a multiple of three iterations the
// result is back in phi, otherwise one copy puts it there.
template <int D, typename T>
static garm_status reinitLoop(cudaStream_t st, const G<D, T> &g, T *phi, T *A, T *B, int iters, double cfl, long long *launches, int *err, bool tune = true) {
	const T dt = T(double(g.dx) * cfl);
	if (iters <= 0) return GARM_OK;
	const ReinitPlan pl = reinitPlanFor<D, T>(st, g, phi, A, dt, err, tune);
	T *buf[3] = {phi, A, B};
	int cur = 0, n = 0;
	for (int it = 0; it < iters; it++) {
		T *u0 = buf[cur], *X = buf[(cur + 1) % 3], *Y = buf[(cur + 2) % 3];
		n += launchReinit<D, T, 0>(pl, st, g, u0, nullptr, X, dt, err);
		n += launchReinit<D, T, 1>(pl, st, g, X, u0, Y, dt, err);
		n += launchReinit<D, T, 2>(pl, st, g, Y, u0, X, dt, err);
		cur = (cur + 1) % 3;
	}
	if (cur != 0 && cudaMemcpyAsync(phi, buf[cur], size_t(g.count()) * sizeof(T), cudaMemcpyDeviceToDevice, st) != cudaSuccess)
		return GARM_CUDA_ERROR;
	if (launches) *launches += n;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status reinitialize(State &s) {
	// fast-marching configuration: FastMarching over a band of 15 cells (LevelSetLiquid.cpp:1151-1152)
	if (s.cfg.fast_marching) return fastMarch<D, T>(s, s.phi, nullptr, 15, s.inStep);
	const G<D, T> g = cellGrid<D, T>(s.geom);
	return reinitLoop<D, T>(s.stream, g, (T *)s.phi, (T *)s.rA, (T *)s.rB, s.cfg.reinit_iters, s.cfg.reinit_cfl, &s.launches, s.reinitErr);
}

// The cached (or freshly tuned) plan of this simulation's grid, for reporting.
template <int D, typename T>
garm_status reinitPlanInfo(State &s, int *form, int *block, int *chunk, float *ms) {
	const G<D, T> g = cellGrid<D, T>(s.geom);
	const ReinitPlan pl = reinitPlanFor<D, T>(s.stream, g, (const T *)s.phi, (T *)s.rA, T(double(g.dx) * s.cfg.reinit_cfl), s.reinitErr);
	*form = pl.form; *block = pl.block; *chunk = pl.chunk; *ms = pl.ms;
	return GARM_OK;
}

template <int D, typename T>
garm_status reinitRaw(cudaStream_t st, const int *size, double dx, T *phi, T *a, T *b, int iters, double cfl, int *err, bool tune) {
	G<D, T> g;
	g.s[0] = size[0]; g.s[1] = size[1]; g.s[2] = D == 3 ? size[2] : 1;
	for (int q = 0; q < 3; q++) g.org[q] = T(0);
	g.dx = T(dx); g.inv = T(1.0 / dx);
	return reinitLoop<D, T>(st, g, phi, a, b, iters, cfl, nullptr, err, tune);
}

// ---------------------------------------------------------------------------
// checkReferenceMap — FP64 arithmetic in every precision mode
// ---------------------------------------------------------------------------
template <int D, typename T>
struct PiPtrs { const T *p[9]; };

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kCheckRefMap(int64_t N, const T *ori, const T *cellDist, PiPtrs<D, T> pi, double band, double threshold, int *counts) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	int tot = 0, bad = 0;
	if (id < N) {
		const double o = double(ori[id]);
		if (fabs(o) < band && double(cellDist[id]) > 0) {
			tot = 1;
			double m[D * D];
#pragma unroll
			for (int q = 0; q < D * D; q++) m[q] = double(pi.p[q][id]);
			auto dot = [&](int p, int q) { double s = m[p * D + 0] * m[q * D + 0]; for (int k = 1; k < D; k++) s = fma(m[p * D + k], m[q * D + k], s); return s; };
			// cos² > θ of a pair of columns, (a·b)²/(|a|²|b|²) > θ, tested as (a·b)² > θ|a|²|b|²:
			// the same decision without the divisions (about ten FP64 instructions each on
			// GB300); a zero column gives false in both forms.
			if (D == 2) {
				const double ab = dot(0, 1);
				if (ab * ab > threshold * (dot(0, 0) * dot(1, 1))) bad = 1;
			} else {
				const double aa = dot(0, 0), bb = dot(1, 1), cc = dot(2, 2);
				const double ab = dot(0, 1), ac = dot(0, 2), bc = dot(1, 2);
				if (ab * ab > threshold * (aa * bb) || ac * ac > threshold * (aa * cc) || bc * bc > threshold * (bb * cc)) bad = 1;
			}
		}
	}
	__shared__ int sh[2][kBlock / 32];
	const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
	for (int o = 16; o > 0; o >>= 1) { tot += __shfl_down_sync(0xffffffffu, tot, o); bad += __shfl_down_sync(0xffffffffu, bad, o); }
	if (lane == 0) { sh[0][w] = tot; sh[1][w] = bad; }
	__syncthreads();
	if (threadIdx.x == 0) {
		int t = 0, b = 0;
		for (int q = 0; q < kBlock / 32; q++) { t += sh[0][q]; b += sh[1][q]; }
		if (t) atomicAdd(counts, t);
		if (b) atomicAdd(counts + 1, b);
	}
}

// restartFlag = !(bad <= ratio * tot): the decision of advance (LevelSetLiquid.cpp:631),
// unless counts[kRestartOverride] holds a decision set by garm_sim_set_restart_override
// (1: keep the reference map, 2: restart).
__global__ void kRestartDecision(const int *counts, double ratio, int *flag, double *stats, const unsigned long long *counter) {
	double *rec = stepRecord(stats, counter);
	const int tot = counts[0], bad = counts[1], force = counts[kRestartOverride];
	const int restart = force == GARM_RESTART_NEVER ? 0 : force == GARM_RESTART_ALWAYS ? 1 : ((1.0 * bad <= ratio * tot) ? 0 : 1);
	*flag = restart;
	if (rec) { rec[kStRestarted] = restart; rec[kStRmTotal] = tot; rec[kStRmBad] = bad; }
}

// Counts and decision on the device, no host synchronisation.
template <int D, typename T>
garm_status checkReferenceMapAsync(State &s, bool record) {
	kClearWords<<<1, 32, 0, s.stream>>>((unsigned *)s.redI32, 2, nullptr, 0); s.launches++;
	PiPtrs<D, T> pp{};
	for (int q = 0; q < D * D; q++) pp.p[q] = (const T *)s.Pi[q];
	kCheckRefMap<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, (const T *)s.ori, (const T *)s.cellDist, pp,
		s.cfg.rm_band * s.geom.dx, s.cfg.rm_threshold, s.redI32); s.launches++;
	kRestartDecision<<<1, 1, 0, s.stream>>>(s.redI32, s.cfg.rm_ratio, s.restartFlag, record ? s.statsDev : nullptr, s.stepCounter); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status checkReferenceMap(State &s, int *keep, int *tot, int *bad) {
	GARM_TRY((checkReferenceMapAsync<D, T>(s, false)));
	int h[2] = {0, 0}, f = 0;
	cudaError_t e = cudaMemcpyAsync(h, s.redI32, sizeof(h), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaMemcpyAsync(&f, s.restartFlag, sizeof(int), cudaMemcpyDeviceToHost, s.stream);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
	if (tot) *tot = h[0];
	if (bad) *bad = h[1];
	if (keep) *keep = f ? 0 : 1;
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// restart (plain branch): φ0 = φ; ψ0 = 4th-order central ∇φ0; ξ = x; Π = I
// ---------------------------------------------------------------------------
template <int D, typename T>
struct RestartIO {
	const T *phi;
	T *ref;
	T *refGrad[3];
	T *xi[3];
	T *Pi[9];
};

template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kRestart(Geom geom, RestartIO<D, T> io, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T *f = io.phi;
	io.ref[id] = f[id];
	const T h = g.inv / T(12);
#pragma unroll
	for (int a = 0; a < D; a++) {
		const int ex = a == 0, ey = a == 1, ez = a == 2;
		const T v0 = ldg(f + g.cidx(i - 2 * ex, j - 2 * ey, k - 2 * ez));
		const T v1 = ldg(f + g.cidx(i - ex, j - ey, k - ez));
		const T v3 = ldg(f + g.cidx(i + ex, j + ey, k + ez));
		const T v4 = ldg(f + g.cidx(i + 2 * ex, j + 2 * ey, k + 2 * ez));
		io.refGrad[a][id] = (v0 - T(8) * v1 + T(8) * v3 - v4) * h;  // Derivatives.h:48
	}
	io.xi[0][id] = g.pos(0, i);
	io.xi[1][id] = g.pos(1, j);
	if (D == 3) io.xi[2][id] = g.pos(2, k);
#pragma unroll
	for (int q = 0; q < D * D; q++) io.Pi[q][id] = (q % (D + 1) == 0) ? T(1) : T(0);
}

// ---------------------------------------------------------------------------
// Newton configuration: restart() by HybridNewton without FMM (LevelSetLiquid.cpp:1290-1308;
// HybridNewton.h:59-127 and 146-467, ENABLE_MODIFIED branch; HybridNewton.cpp:30-118).
// Every kernel takes the restart gate, so the branch can sit inside a captured step.
// ---------------------------------------------------------------------------
template <int D, typename T>
struct NewtonIO {
	const T *phi;                 // the reinitialised level set (starting points)
	T *ori, *lsGrad[3];           // HybridNewton's φ and ∇φ (in: _oriLevelSet, _levelSetGrad)
	T *hp, *hg[3];                // second buffer of φ and ∇φ
	T *mixed[4];                  // Hermite mixed derivatives of the current ∇φ
	T *pts[3];                    // starting points of the closest-point search
	uint8_t *mark0, *mark1;       // cells next to a sign change, and one more layer
	T *ref, *refGrad[3];          // outputs: _refLevelSet, _refLevelSetGrad
	T *xi[3], *Pi[9];             // ξ = x, Π = I
};

// ScalarFieldWrapper::gradient (ScalarField.h:41-47): the trilinear blend of the central
// differences (Derivatives.h:47-57) at the 2^D samples around p.
template <int D, typename T>
__device__ __forceinline__ void blendGradient(const G<D, T> &g, const T *f, const T *pos, T *gr) {
	int ll[3] = {0, 0, 0};
	T fr[3] = {T(0), T(0), T(0)};
#pragma unroll
	for (int a = 0; a < D; a++) { ll[a] = g.lower(a, pos[a]); fr[a] = g.frac(a, pos[a], ll[a]); }
	const T h = T(0.5) * g.inv;
	for (int q = 0; q < (1 << D); q++) {
		const int n[3] = {ll[0] + (q & 1), ll[1] + (q >> 1 & 1), D == 3 ? ll[2] + (q >> 2 & 1) : 0};
		T wt = T(1);
#pragma unroll
		for (int a = 0; a < D; a++) wt *= ((q >> a) & 1) ? fr[a] : T(1) - fr[a];
#pragma unroll
		for (int a = 0; a < D; a++) {
			const int ex = a == 0, ey = a == 1, ez = a == 2;
			const T d = (ldg(f + g.cidx(n[0] + ex, n[1] + ey, n[2] + ez)) - ldg(f + g.cidx(n[0] - ex, n[1] - ey, n[2] - ez))) * h;
			gr[a] += d * wt;
		}
	}
}

// Starting points p − φ(p)·∇φ(p) from _levelSetView: the cubic Lagrange value and, as
// ScalarFieldWrapper::gradient does, the trilinear blend of the central differences at
// the eight surrounding samples (ScalarField.h:41-47, Derivatives.h:47-57).
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnPoints(Geom geom, NewtonIO<D, T> io, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int ci, cj, ck;
	g.coord(id, ci, cj, ck);
	const T pos[3] = {g.pos(0, ci), g.pos(1, cj), D == 3 ? g.pos(2, ck) : T(0)};
	const T *f = io.phi;
	// cubic value (CubicIntrpl, LagrangeIntrpl.h:137-170)
	int cl[3] = {0, 0, 0};
	T w[3][4];
	const T sixth = T(1.0 / 6.0);
#pragma unroll
	for (int a = 0; a < D; a++) {
		cl[a] = g.lower(a, pos[a]) - 1;
		const T x = g.frac(a, pos[a], cl[a]);
		const T x1 = x - T(1), x2 = x - T(2), x3 = x - T(3);
		w[a][0] = -(x1 * x2 * x3) * sixth;
		w[a][1] = x * x2 * x3 * T(0.5);
		w[a][2] = -(x * x1 * x3) * T(0.5);
		w[a][3] = x * x1 * x2 * sixth;
	}
	T v = T(0);
	for (int c = 0; c < (D == 3 ? 4 : 1); c++) {
		T sy = T(0);
		for (int b = 0; b < 4; b++) {
			T sx = T(0);
#pragma unroll
			for (int a = 0; a < 4; a++) sx += ldg(f + g.cidx(cl[0] + a, cl[1] + b, D == 3 ? cl[2] + c : 0)) * w[0][a];
			sy += sx * w[1][b];
		}
		v += D == 3 ? sy * w[2][c] : sy;
	}
	T gr[3] = {T(0), T(0), T(0)};
	blendGradient<D, T>(g, f, pos, gr);
#pragma unroll
	for (int a = 0; a < D; a++) io.pts[a][id] = pos[a] - v * gr[a];
}

// prepareInterface (HybridNewton.cpp:59-75): cells with a sign change (φ·φ_nb <= 0) to a neighbour.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnMark(Geom geom, const T *phi, uint8_t *mark, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T f = phi[id];
	uint8_t m = 0;
	for (int nb = 0; nb < 2 * D && !m; nb++) {
		const int a = nb >> 1, s = (nb & 1) ? 1 : -1;
		const int ni = i + (a == 0 ? s : 0), nj = j + (a == 1 ? s : 0), nk = k + (a == 2 ? s : 0);
		if (g.valid(ni, nj, nk) && f * phi[g.idx(ni, nj, nk)] <= T(0)) m = 1;
	}
	mark[id] = m;
}

// extrapolate(1) (HybridNewton.cpp:96-118): one more layer of marked cells.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnDilate(Geom geom, const uint8_t *in, uint8_t *out, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	uint8_t m = in[id];
	for (int nb = 0; nb < 2 * D && !m; nb++) {
		const int a = nb >> 1, s = (nb & 1) ? 1 : -1;
		const int ni = i + (a == 0 ? s : 0), nj = j + (a == 1 ? s : 0), nk = k + (a == 2 ? s : 0);
		if (g.valid(ni, nj, nk) && in[g.idx(ni, nj, nk)]) m = 1;
	}
	out[id] = m;
}

// v/|v|, or (for the velocity of the eikonal trace) the x unit vector when v = 0;
// normalized() of a zero vector is the zero vector.
template <int D, typename T>
__device__ __forceinline__ void normalizeOr(T *v, bool unitIfZero) {
	T n2 = T(0);
#pragma unroll
	for (int a = 0; a < D; a++) n2 = fma(v[a], v[a], n2);
	if (n2 > T(0)) {
		const T n = sqrt(n2);
#pragma unroll
		for (int a = 0; a < D; a++) v[a] = v[a] / n;
	} else if (unitIfZero) {
		v[0] = T(1);
	}
}

// initializeInterface with the given starting points (HybridNewton.h:102-127): on marked
// cells the modified Newton closest point (HybridNewton.h:146-467): 20 steps of
// delta = -φ ψ/|ψ|² + (s - x) - ψ ((s - x)·ψ)/|ψ|², each at most 0.9 dx long, stopping
// after a step shorter than 1e-3 dx² (2D) or 1e-3 dx³ (3D); φ = ±|s - x|, ψ = ∇H(x)/|∇H(x)|.
// Unmarked cells are copied.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnInterface(Geom geom, NewtonIO<D, T> io, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	const T f = io.ori[id];
	if (!io.mark1[id]) {
		io.hp[id] = f;
#pragma unroll
		for (int a = 0; a < D; a++) io.hg[a][id] = io.lsGrad[a][id];
		return;
	}
	int ci, cj, ck;
	g.coord(id, ci, cj, ck);
	const T start[3] = {g.pos(0, ci), g.pos(1, cj), D == 3 ? g.pos(2, ck) : T(0)};
	T pos[3] = {io.pts[0][id], io.pts[1][id], D == 3 ? io.pts[2][id] : T(0)};
	const T dx = g.dx;
	const T tolerance = T(1e-3) * dx * dx * (D == 2 ? T(1) : dx);
	const T radius = T(0.9) * dx;
	const T *const grad[3] = {io.lsGrad[0], io.lsGrad[1], io.lsGrad[2]};
	const T *const mixed[4] = {io.mixed[0], io.mixed[1], io.mixed[2], io.mixed[3]};
	for (int iter = 0; iter < 20; iter++) {
		T phiv, psi[3] = {T(0), T(0), T(0)};
		hermiteValueGrad<D, T>(g, pos, io.ori, grad, mixed, phiv, psi);
		T s2 = T(0), dot = T(0);
#pragma unroll
		for (int a = 0; a < D; a++) { s2 = fma(psi[a], psi[a], s2); dot = fma(start[a] - pos[a], psi[a], dot); }
		T delta[3], n2 = T(0);
#pragma unroll
		for (int a = 0; a < D; a++) {
			delta[a] = -phiv * psi[a] / s2 + ((start[a] - pos[a]) - psi[a] * dot / s2);
			n2 = fma(delta[a], delta[a], n2);
		}
		T norm = sqrt(n2);
		if (norm > radius) {
#pragma unroll
			for (int a = 0; a < D; a++) delta[a] *= radius / norm;
			norm = radius;
		}
#pragma unroll
		for (int a = 0; a < D; a++) pos[a] += delta[a];
		if (norm < tolerance) break;
	}
	T d2 = T(0);
#pragma unroll
	for (int a = 0; a < D; a++) d2 = fma(start[a] - pos[a], start[a] - pos[a], d2);
	io.hp[id] = sqrt(d2) * (f < T(0) ? T(-1) : T(1));
	T v, gr[3] = {T(0), T(0), T(0)};
	hermiteValueGrad<D, T>(g, pos, io.ori, grad, mixed, v, gr);
	normalizeOr<D, T>(gr, false);
#pragma unroll
	for (int a = 0; a < D; a++) io.hg[a][id] = gr[a];
}

// One step of HybridNewton::advect (HybridNewton.cpp:30-48) on unmarked cells: a TVD-RK3
// trace (Advection.h:44-49) along the normalised ∇H for -sgn·dt, then φ = H(x) + sgn·dt,
// ψ = ∇H(x)/|∇H(x)|.  Marked cells are copied.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnAdvect(Geom geom, const T *fin, const T *g0, const T *g1, const T *g2, NewtonIO<D, T> io,
                                                    T *fout, T *o0, T *o1, T *o2, T dt, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	const T *const grad[3] = {g0, g1, g2};
	T *const gout[3] = {o0, o1, o2};
	const T f = fin[id];
	if (io.mark1[id]) {
		fout[id] = f;
#pragma unroll
		for (int a = 0; a < D; a++) gout[a][id] = grad[a][id];
		return;
	}
	const T *const mixed[4] = {io.mixed[0], io.mixed[1], io.mixed[2], io.mixed[3]};
	int ci, cj, ck;
	g.coord(id, ci, cj, ck);
	const T pos[3] = {g.pos(0, ci), g.pos(1, cj), D == 3 ? g.pos(2, ck) : T(0)};
	const T sgn = f < T(0) ? T(-1) : T(1);
	const T h = -sgn * dt;
	auto vel = [&](const T *p, T *out) {
		T v;
		out[0] = out[1] = out[2] = T(0);
		hermiteValueGrad<D, T>(g, p, fin, grad, mixed, v, out);
		normalizeOr<D, T>(out, true);
	};
	T v0[3], v1[3], v2[3], p1[3] = {T(0), T(0), T(0)}, p2[3] = {T(0), T(0), T(0)}, tp[3] = {T(0), T(0), T(0)};
	vel(pos, v0);
#pragma unroll
	for (int a = 0; a < D; a++) p1[a] = pos[a] + v0[a] * h;
	vel(p1, v1);
#pragma unroll
	for (int a = 0; a < D; a++) p2[a] = pos[a] + (v0[a] + v1[a]) * h / T(4);
	vel(p2, v2);
#pragma unroll
	for (int a = 0; a < D; a++) tp[a] = pos[a] + (v0[a] + v1[a] + T(4) * v2[a]) * h / T(6);
	T val, gr[3] = {T(0), T(0), T(0)};
	hermiteValueGrad<D, T>(g, tp, fin, grad, mixed, val, gr);
	fout[id] = val + sgn * dt;
	normalizeOr<D, T>(gr, false);
#pragma unroll
	for (int a = 0; a < D; a++) gout[a][id] = gr[a];
}

// The end of HybridNewton::sweep (HybridNewton.cpp:56-63): on unmarked cells ψ is the
// normalised gradient of the cubic view of the marched φ.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnSweepGrad(Geom geom, NewtonIO<D, T> io, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count() || io.mark1[id]) return;
	int ci, cj, ck;
	g.coord(id, ci, cj, ck);
	const T pos[3] = {g.pos(0, ci), g.pos(1, cj), D == 3 ? g.pos(2, ck) : T(0)};
	T gr[3] = {T(0), T(0), T(0)};
	blendGradient<D, T>(g, io.hp, pos, gr);
	normalizeOr<D, T>(gr, false);
#pragma unroll
	for (int a = 0; a < D; a++) io.hg[a][id] = gr[a];
}

// The result into _oriLevelSet/_levelSetGrad and _refLevelSet/_refLevelSetGrad; ξ = x, Π = I.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kHnFinish(Geom geom, NewtonIO<D, T> io, const int *gate) {
	if (gate && !*gate) return;
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T f = io.hp[id];
	io.ori[id] = f;
	io.ref[id] = f;
#pragma unroll
	for (int a = 0; a < D; a++) { const T v = io.hg[a][id]; io.lsGrad[a][id] = v; io.refGrad[a][id] = v; }
	io.xi[0][id] = g.pos(0, i);
	io.xi[1][id] = g.pos(1, j);
	if (D == 3) io.xi[2][id] = g.pos(2, k);
#pragma unroll
	for (int q = 0; q < D * D; q++) io.Pi[q][id] = (q % (D + 1) == 0) ? T(1) : T(0);
}

template <int D, typename T>
static garm_status newtonRestart(State &s) {
	NewtonIO<D, T> io{};
	io.phi = (const T *)s.phi;
	io.ori = (T *)s.ori; io.hp = (T *)s.hnPhi; io.ref = (T *)s.ref;
	for (int a = 0; a < D; a++) {
		io.lsGrad[a] = (T *)s.lsGrad[a]; io.hg[a] = (T *)s.hnGrad[a]; io.pts[a] = (T *)s.hnPoints[a];
		io.refGrad[a] = (T *)s.refGrad[a]; io.xi[a] = (T *)s.xi[a];
	}
	for (int q = 0; q < 4; q++) io.mixed[q] = (T *)s.hnMixed[q];
	for (int q = 0; q < D * D; q++) io.Pi[q] = (T *)s.Pi[q];
	io.mark0 = s.hnMark[0]; io.mark1 = s.hnMark[1];
	const unsigned nb = gridFor(s.N);
	kHnPoints<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
	kHnMark<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io.ori, io.mark0, s.gate); s.launches++;
	kHnDilate<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io.mark0, io.mark1, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	GARM_TRY((scalarMixed<D, T>(s, io.lsGrad, io.mixed)));
	kHnInterface<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	if (s.cfg.fast_marching) {
		// sweep, maxSteps 20 (HybridNewton.cpp:51-64): fast marching from the marked cells
		GARM_TRY((fastMarch<D, T>(s, io.hp, io.mark1, 20, s.inStep)));
		kHnSweepGrad<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
		GARM_CHECK_LAUNCH();
		kHnFinish<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
		GARM_CHECK_LAUNCH();
		return resetRefView<D, T>(s);
	}
	// advect, maxSteps 20, cfl 0.9 (LevelSetLiquid.cpp:1301): the buffers alternate, so after
	// an even number of steps the result is back in (hp, hg)
	const T dt = T(s.geom.dx * 0.9);
	for (int it = 0; it < 20; it++) {
		const bool fromH = (it & 1) == 0;
		T *fin = fromH ? io.hp : io.ori, *fout = fromH ? io.ori : io.hp;
		T *const *gin = fromH ? io.hg : io.lsGrad;
		T *const *gout = fromH ? io.lsGrad : io.hg;
		GARM_TRY((scalarMixed<D, T>(s, gin, io.mixed)));
		kHnAdvect<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, fin, gin[0], gin[1], D == 3 ? gin[2] : gin[0], io, fout, gout[0], gout[1],
		                                             D == 3 ? gout[2] : gout[0], dt, s.gate); s.launches++;
		GARM_CHECK_LAUNCH();
	}
	kHnFinish<D, T><<<nb, kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return resetRefView<D, T>(s);
}

template <int D, typename T>
garm_status restart(State &s) {
	if (s.cfg.restart_newton) return newtonRestart<D, T>(s);
	RestartIO<D, T> io{};
	io.phi = (const T *)s.phi;
	io.ref = (T *)s.ref;
	for (int a = 0; a < D; a++) { io.refGrad[a] = (T *)s.refGrad[a]; io.xi[a] = (T *)s.xi[a]; }
	for (int q = 0; q < D * D; q++) io.Pi[q] = (T *)s.Pi[q];
	kRestart<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, io, s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return resetRefView<D, T>(s);
}

// ψ0 = computeFirst<4>(φ0) as loadFrame does without Newton (LevelSetLiquid.cpp:507-509)
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kRefGrad4(Geom geom, const T *ref, T *g0, T *g1, T *g2) {
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	T *out[3] = {g0, g1, g2};
	const T h = g.inv / T(12);
#pragma unroll
	for (int a = 0; a < D; a++) {
		const int ex = a == 0, ey = a == 1, ez = a == 2;
		const T v0 = ldg(ref + g.cidx(i - 2 * ex, j - 2 * ey, k - 2 * ez));
		const T v1 = ldg(ref + g.cidx(i - ex, j - ey, k - ez));
		const T v3 = ldg(ref + g.cidx(i + ex, j + ey, k + ez));
		const T v4 = ldg(ref + g.cidx(i + 2 * ex, j + 2 * ey, k + 2 * ez));
		out[a][id] = (v0 - T(8) * v1 + T(8) * v3 - v4) * h;
	}
}

// ∇φ of the level set, computeFirst<4>(_levelSet, _levelSetGrad) (LevelSetLiquid.cpp:546-548)
template <int D, typename T>
garm_status levelSetGradient(State &s) {
	kRefGrad4<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, (const T *)s.phi, (T *)s.lsGrad[0], (T *)s.lsGrad[1], (T *)(D == 3 ? s.lsGrad[2] : nullptr)); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status refreshRefGradient(State &s) {
	kRefGrad4<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, (const T *)s.ref, (T *)s.refGrad[0], (T *)s.refGrad[1], (T *)(D == 3 ? s.refGrad[2] : nullptr)); s.launches++;
	GARM_CHECK_LAUNCH();
	return resetRefView<D, T>(s);
}

// ξ = x, advRegion = 1, Π = I (LevelSetLiquid.cpp:560-566)
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kInitRefMap(Geom geom, RestartIO<D, T> io, uint8_t *adv) {
	const G<D, T> g = cellGrid<D, T>(geom);
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	io.xi[0][id] = g.pos(0, i);
	io.xi[1][id] = g.pos(1, j);
	if (D == 3) io.xi[2][id] = g.pos(2, k);
#pragma unroll
	for (int q = 0; q < D * D; q++) io.Pi[q][id] = (q % (D + 1) == 0) ? T(1) : T(0);
	adv[id] = 1;
}

template <int D, typename T>
garm_status initRefMap(State &s) {
	RestartIO<D, T> io{};
	for (int a = 0; a < D; a++) io.xi[a] = (T *)s.xi[a];
	for (int q = 0; q < D * D; q++) io.Pi[q] = (T *)s.Pi[q];
	kInitRefMap<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, io, s.adv); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// enforceBoundaryLevelSet(sdf, tol): sdf = max(sdf, -cellDist - tol)
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kBlock) kEnforceBoundaryLevelSet(int64_t N, T *sdf, const T *cellDist, T tol) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= N) return;
	const T lim = -cellDist[id] - tol;
	if (sdf[id] < lim) sdf[id] = lim;
}

template <int D, typename T>
garm_status enforceBoundaryLevelSet(State &s, void *field, double tol) {
	kEnforceBoundaryLevelSet<T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.N, (T *)field, (const T *)s.cellDist, T(tol)); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

#define GARM_INST(D, T) \
	template garm_status generateCurrentFields<D, T>(State &); \
	template garm_status reinitialize<D, T>(State &); \
	template garm_status reinitPlanInfo<D, T>(State &, int *, int *, int *, float *); \
	template garm_status reinitRaw<D, T>(cudaStream_t, const int *, double, T *, T *, T *, int, double, int *, bool); \
	template garm_status checkReferenceMap<D, T>(State &, int *, int *, int *); \
	template garm_status checkReferenceMapAsync<D, T>(State &, bool); \
	template garm_status restart<D, T>(State &); \
	template garm_status initRefMap<D, T>(State &); \
	template garm_status refreshRefGradient<D, T>(State &); \
	template garm_status levelSetGradient<D, T>(State &); \
	template garm_status enforceBoundaryLevelSet<D, T>(State &, void *, double);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
