// garm_levelset.cu — level-set stages of LevelSetLiquid::advance:
//   generateCurrentFields   (Source/Core/LevelSetLiquid.cpp:1218-1244)
//   reinitializeLevelSet    (LevelSetLiquid.cpp:1148-1160 → Reinitialization.h:20-80, Derivatives.h:134-159)
//   checkReferenceMap       (LevelSetLiquid.cpp:1246-1283)
//   restart, plain branch   (LevelSetLiquid.cpp:1320-1352)
//   enforceBoundaryLevelSet (LevelSetLiquid.cpp:966-975)
#include "garm_internal.h"

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
};

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
	T phi = hermiteScalar<D, T>(g, p, io.ref, io.refGrad, io.refMixed);
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
	const double airClamp = s.cfg.air_extrap_radius * s.geom.dx;
	kCompose<D, T><<<gridFor(s.N), kBlock, 0, s.stream>>>(s.geom, io, T(airClamp), T(3.0 * s.geom.dx), s.gate); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

// ---------------------------------------------------------------------------
// WENO5 reinitialisation (Reinitialization.h:20-80)
// ---------------------------------------------------------------------------
// 2^-e for the binary exponent e of x > 0 (x normal): an exact power-of-two
// scale built from the exponent bits, used to keep the WENO weights in range.
__device__ __forceinline__ double pow2NegExp(double x) {
	const int hi = __double2hiint(x);
	const int e = ((hi >> 20) & 0x7ff) - 1023;
	return __hiloint2double((1023 - e) << 20, 0);
}
__device__ __forceinline__ float pow2NegExp(float x) {
	const int e = ((__float_as_int(x) >> 23) & 0xff) - 127;
	return __int_as_float((127 - e) << 23);
}

// One one-sided WENO5 derivative from five differences (Derivatives.h:137-157),
// returned without the 1/(6 dx) factor.  The three weights α_k = d_k/(s_k+ε)^2 are
// normalised with a single division: with q_k = (s_k+ε)·2^-e (2^e ~ ε, an exact
// scale) every q_k lies in [1/2, ~7e7], so d_k·q_i^2·q_j^2 neither overflows nor
// underflows in FP32 or FP64, and Σα_k P_k / Σα_k = Σ w_k P_k / Σ w_k with
// w_1 = .1 q_2^2 q_3^2, w_2 = .6 q_1^2 q_3^2, w_3 = .3 q_1^2 q_2^2.
template <typename T>
__device__ __forceinline__ T wenoSide(T d0, T d1, T d2, T d3, T d4, T sq0, T sq1, T sq2, T sq3, T sq4, T floorEps) {
	const T m = fmax(fmax(fmax(sq0, sq1), fmax(sq2, sq3)), sq4);
	const T eps = fma(m, T(1e-6), floorEps);
	const T P1 = T(2) * d0 - T(7) * d1 + T(11) * d2;   // 6·phix1
	const T P2 = -d1 + T(5) * d2 + T(2) * d3;           // 6·phix2
	const T P3 = T(2) * d2 + T(5) * d3 - d4;            // 6·phix3
	const T e1 = d0 - T(2) * d1 + d2, f1 = d0 - T(4) * d1 + T(3) * d2;
	const T e2 = d1 - T(2) * d2 + d3, f2 = d1 - d3;
	const T e3 = d2 - T(2) * d3 + d4, f3 = T(3) * d2 - T(4) * d3 + d4;
	const T c13 = T(13.0 / 12.0);
	const T s1 = fma(c13 * e1, e1, T(0.25) * f1 * f1);
	const T s2 = fma(c13 * e2, e2, T(0.25) * f2 * f2);
	const T s3 = fma(c13 * e3, e3, T(0.25) * f3 * f3);
	const T sc = pow2NegExp(eps);
	const T q1 = (s1 + eps) * sc, q2 = (s2 + eps) * sc, q3 = (s3 + eps) * sc;
	const T t1 = q1 * q1, t2 = q2 * q2, t3 = q3 * q3;
	const T w1 = T(0.1) * t2 * t3, w2 = T(0.6) * t1 * t3, w3 = T(0.3) * t1 * t2;
	return (w1 * P1 + w2 * P2 + w3 * P3) / (w1 + w2 + w3);
}

// weno5 (Derivatives.h:134-159): one-sided derivatives (φ⁻, φ⁺) from seven values.
template <typename T>
__device__ __forceinline__ void weno5(const T v[7], T invDx, T &dm, T &dp) {
	// 1e-99 in FP64 (Derivatives.h:144); FP32 takes the smallest comparable normal number
	const T floorEps = sizeof(T) == 8 ? T(1e-99) : T(1e-30);
	const T D1 = v[1] - v[0], D2 = v[2] - v[1], D3 = v[3] - v[2], D4 = v[4] - v[3], D5 = v[5] - v[4], D6 = v[6] - v[5];
	const T Q1 = D1 * D1, Q2 = D2 * D2, Q3 = D3 * D3, Q4 = D4 * D4, Q5 = D5 * D5, Q6 = D6 * D6;
	const T k = invDx * T(1.0 / 6.0);
	dm = wenoSide<T>(D1, D2, D3, D4, D5, Q1, Q2, Q3, Q4, Q5, floorEps) * k;
	dp = wenoSide<T>(D6, D5, D4, D3, D2, Q6, Q5, Q4, Q3, Q2, floorEps) * k;
}

// One TVD-RK3 sub-stage: out = lin(base, in + dt*L(in)).
// mode 0: out = adv;  mode 1: out = (3*base + adv)/4;  mode 2: out = (base + 2*adv)/3.
template <int D, typename T, int Mode>
__global__ void __launch_bounds__(kBlock) kReinitStage(G<D, T> g, const T *__restrict__ in, const T *base, T *out, T dt) {
	const int64_t id = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
	if (id >= g.count()) return;
	int i, j, k;
	g.coord(id, i, j, k);
	const T f = ldg(in + id);
	// Stencil addressing: the base of the line through the cell along each axis,
	// plus one clamped coordinate per load (clamp-to-edge, GridBasedData.h:47).
	const int sx = g.s[0], sy = g.s[1], sz = D == 3 ? g.s[2] : 1;
	const int sxy = sx * sy;
	const T *line[3] = {in + (id - i), in + (id - j * sx), in + (id - k * sxy)};
	const int lim[3] = {sx - 1, sy - 1, sz - 1};
	const int pos[3] = {i, j, k};
	const int str[3] = {1, sx, sxy};
	T sum = T(0);
#pragma unroll
	for (int a = 0; a < D; a++) {
		T v[7];
#pragma unroll
		for (int t = 0; t < 7; t++) v[t] = ldg(line[a] + min(max(pos[a] + t - 3, 0), lim[a]) * str[a]);
		T dm, dp;
		weno5<T>(v, g.inv, dm, dp);
		if (f < T(0)) { const T x = fmin(dm, T(0)), y = fmax(dp, T(0)); sum += x * x; sum += y * y; }
		else { const T x = fmax(dm, T(0)), y = fmin(dp, T(0)); sum += x * x; sum += y * y; }
	}
	sum = sqrt(sum);
	const T sp = g.dx * sum;
	const T sgn = f * rsqrt(f * f + sp * sp);  // smoothed sign (Reinitialization.h:26)
	const T adv = f + dt * sgn * (T(1) - sum);
	T r;
	if (Mode == 0) r = adv;
	else if (Mode == 1) r = (base[id] * T(3) + adv) / T(4);
	else r = (base[id] + adv * T(2)) / T(3);
	out[id] = r;
}

template <int D, typename T>
static garm_status reinitLoop(cudaStream_t st, const G<D, T> &g, T *phi, T *A, T *B, int iters, double cfl, long long *launches) {
	const T dt = T(double(g.dx) * cfl);
	const unsigned nb = gridFor(g.count());
	for (int it = 0; it < iters; it++) {
		kReinitStage<D, T, 0><<<nb, kBlock, 0, st>>>(g, phi, nullptr, A, dt);
		kReinitStage<D, T, 1><<<nb, kBlock, 0, st>>>(g, A, phi, B, dt);
		kReinitStage<D, T, 2><<<nb, kBlock, 0, st>>>(g, B, phi, phi, dt);
		if (launches) *launches += 3;
	}
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

template <int D, typename T>
garm_status reinitialize(State &s) {
	const G<D, T> g = cellGrid<D, T>(s.geom);
	return reinitLoop<D, T>(s.stream, g, (T *)s.phi, (T *)s.rA, (T *)s.rB, s.cfg.reinit_iters, s.cfg.reinit_cfl, &s.launches);
}

template <int D, typename T>
garm_status reinitRaw(cudaStream_t st, const int *size, double dx, T *phi, T *a, T *b, int iters, double cfl) {
	G<D, T> g;
	g.s[0] = size[0]; g.s[1] = size[1]; g.s[2] = D == 3 ? size[2] : 1;
	for (int q = 0; q < 3; q++) g.org[q] = T(0);
	g.dx = T(dx); g.inv = T(1.0 / dx);
	return reinitLoop<D, T>(st, g, phi, a, b, iters, cfl, nullptr);
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
			if (D == 2) {
				const double ab = dot(0, 1);
				if (ab * ab / dot(0, 0) / dot(1, 1) > threshold) bad = 1;
			} else {
				const double aa = dot(0, 0), bb = dot(1, 1), cc = dot(2, 2);
				const double ab = dot(0, 1), ac = dot(0, 2), bc = dot(1, 2);
				const double vab = ab * ab / aa / bb, vac = ac * ac / aa / cc, vbc = bc * bc / bb / cc;
				if (vab > threshold || vac > threshold || vbc > threshold) bad = 1;
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

// restartFlag = !(bad <= ratio * tot): the decision of advance (LevelSetLiquid.cpp:631)
__global__ void kRestartDecision(const int *counts, double ratio, int *flag, double *stats, const unsigned long long *counter) {
	double *rec = stepRecord(stats, counter);
	const int tot = counts[0], bad = counts[1];
	const int restart = (1.0 * bad <= ratio * tot) ? 0 : 1;
	*flag = restart;
	if (rec) { rec[kStRestarted] = restart; rec[kStRmTotal] = tot; rec[kStRmBad] = bad; }
}

// Counts and decision on the device, no host synchronisation.
template <int D, typename T>
garm_status checkReferenceMapAsync(State &s, bool record) {
	cudaError_t e = cudaMemsetAsync(s.redI32, 0, 2 * sizeof(int), s.stream);
	if (e != cudaSuccess) return GARM_CUDA_ERROR;
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

template <int D, typename T>
garm_status restart(State &s) {
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
	template garm_status reinitRaw<D, T>(cudaStream_t, const int *, double, T *, T *, T *, int, double); \
	template garm_status checkReferenceMap<D, T>(State &, int *, int *, int *); \
	template garm_status checkReferenceMapAsync<D, T>(State &, bool); \
	template garm_status restart<D, T>(State &); \
	template garm_status initRefMap<D, T>(State &); \
	template garm_status refreshRefGradient<D, T>(State &); \
	template garm_status enforceBoundaryLevelSet<D, T>(State &, void *, double);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
