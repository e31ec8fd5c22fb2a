// garm_volume.cu — LevelSetLiquid::calculateVolume (Source/Core/LevelSetLiquid.cpp:1162-1190),
// the liquid-volume diagnostic kept outside the timed step:
//   2D: area of the filled marching-squares contour of tmp (Contourer<2,true>, Contourer.cpp:10-96)
//   3D: sum over the cubes between samples of the marching-cubes-style volume of Takahashi &
//       Batty, "Fast Marching-Cubes-Style Volume Evaluation for Level Set Surfaces", JCGT 11(2),
//       2022 (the reference's copy: MC-style-vol-eval/fraction.hpp:149-775).
// One thread per cube (grid-stride over a fixed grid), FP64 arithmetic in both precision
// forms, per-block sums and a fixed-order final sum: the result does not depend on scheduling.
#include "garm_internal.h"

#include <algorithm>
#include <mutex>

namespace garm {
namespace {

// ---- tables (built on the host once per device, copied to constant memory) ----
// Evaluator corner order: (0,0,0), (1,0,0), (1,1,0), (0,1,0), (0,0,1), (1,0,1), (1,1,1), (0,1,1).
constexpr int kCorner[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
// Inside pattern (bit i: corner i below zero) of each of the 23 canonical cases.
constexpr int kCanonical[23] = {0, 1, 3, 33, 65, 14, 67, 82, 15, 141, 170, 77, 30, 90, 142, 173, 188, 241, 190, 222, 252, 254, 255};
// Rotation that brings each inside pattern to its canonical case ('A' + index into the
// rotation list built below, pattern 0 first).  Where several rotations do, the choice
// fixes the triangulation the closed form integrates, so it is the evaluator's
// (fraction.hpp:510-767) expressed in this list's order.
constexpr char kRotation[257] =
	"AACAKIIDLDLKKTAABGRXKRIKDJIPKTANHAXBXRMFHDXKLTFHBQGXBQGWHXGLMEOO"
	"OASAMMFFMVXKUAOSBGAXWDFPKJABUCDJFSIGCCIVFBINCJPNEQNOIURPETMEQCUE"
	"EUCQEMTDPRUTOAAENPJXNPXFVRVCRISFJDCBBPMKPRAWOAGBSXQUSXVMSFMMASAO"
	"OOEILLCHWRWBLGQBHSHLLXDHRMRXBXAHNNIKIIJDLIRKXRGBSATKKLDLDIIKACAA";

struct McTables {
	unsigned char perm[256][8];  // per pattern: rotated corner i takes the value of corner perm[i]
	unsigned char kase[256];     // canonical case, +32 for the second triangulation of case 9
};
__constant__ McTables c_mc;

bool buildTables(McTables &t) {
	int perms[24][8];
	auto cornerIndex = [](int x, int y, int z) {
		for (int i = 0; i < 8; i++) if (kCorner[i][0] == x && kCorner[i][1] == y && kCorner[i][2] == z) return i;
		return -1;
	};
	// the 24 proper rotations: closure of the identity under quarter turns about the
	// three axes through the centre, breadth first
	int n = 1;
	for (int i = 0; i < 8; i++) perms[0][i] = i;
	for (int k = 0; k < n; k++)
		for (int axis = 0; axis < 3; axis++) {
			int q[8];
			for (int i = 0; i < 8; i++) {
				int c[3] = {kCorner[i][0], kCorner[i][1], kCorner[i][2]};
				const int a = (axis + 1) % 3, b = (axis + 2) % 3;
				const int na = c[b], nb = 1 - c[a];
				c[a] = na; c[b] = nb;
				q[i] = perms[k][cornerIndex(c[0], c[1], c[2])];
			}
			bool seen = false;
			for (int m = 0; m < n && !seen; m++) seen = std::equal(q, q + 8, perms[m]);
			if (!seen && n < 24) { std::copy(q, q + 8, perms[n]); n++; }
		}
	if (n != 24) return false;
	for (int p = 0; p < 256; p++) {
		const int r = kRotation[p] - 'A';
		if (r < 0 || r >= 24) return false;
		int q = 0;
		for (int i = 0; i < 8; i++) { t.perm[p][i] = (unsigned char)perms[r][i]; if (p >> perms[r][i] & 1) q |= 1 << i; }
		int c = -1;
		for (int k = 0; k < 23; k++) if (kCanonical[k] == q) c = k;
		if (c < 0) return false;
		t.kase[p] = (unsigned char)(c + ((c == 9 && (p & 2)) ? 32 : 0));  // case 9: corner 1 inside -> second form
	}
	return true;
}

std::mutex g_tableMutex;
bool g_tablesOn[64] = {};

garm_status ensureTables() {
	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return GARM_CUDA_ERROR; }
	std::lock_guard<std::mutex> lock(g_tableMutex);
	if (g_tablesOn[dev]) return GARM_OK;
	static McTables host;
	static bool built = false, ok = false;
	if (!built) { ok = buildTables(host); built = true; }
	if (!ok) return GARM_NUMERIC;
	if (cudaMemcpyToSymbol(c_mc, &host, sizeof(McTables)) != cudaSuccess) { cudaGetLastError(); return GARM_CUDA_ERROR; }
	g_tablesOn[dev] = true;
	return GARM_OK;
}

// ---- per-cell pieces ----
// Edges as (corner at coordinate 0, corner at coordinate 1) along one axis.
__constant__ unsigned char c_edge[12][2] = {{0, 1}, {1, 2}, {3, 2}, {0, 3}, {4, 5}, {5, 6}, {7, 6}, {4, 7}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
// Coordinates of corner i in the evaluator's order (kCorner).
__device__ __forceinline__ double cornerX(int i) { const int r = i & 3; return (r == 1 || r == 2) ? 1.0 : 0.0; }
__device__ __forceinline__ double cornerY(int i) { return (i & 3) >= 2 ? 1.0 : 0.0; }
__device__ __forceinline__ double cornerZ(int i) { return i >= 4 ? 1.0 : 0.0; }
// Fraction of edge a-b below zero, measured from its inside end (fraction.hpp:56-61).
__device__ __forceinline__ double insideFrac(double a, double b) {
	if (a < 0 && b < 0) return 1.0;
	if (a < 0) return a / (a - b);
	if (b < 0) return b / (b - a);
	return 0.0;
}

// (p1 - p0) x (p0 - p2) . p0: six times a signed tetrahedron volume, in the
// orientation the closed forms use.
__device__ __forceinline__ double sv(const double *p0, const double *p1, const double *p2) {
	const double u0 = p1[0] - p0[0], u1 = p1[1] - p0[1], u2 = p1[2] - p0[2];
	const double w0 = p0[0] - p2[0], w1 = p0[1] - p2[1], w2 = p0[2] - p2[2];
	return (u1 * w2 - u2 * w1) * p0[0] + (u2 * w0 - u0 * w2) * p0[1] + (u0 * w1 - u1 * w0) * p0[2];
}

struct Cube {
	double v[8];
	__device__ double f(int a, int b) const { return insideFrac(v[a], v[b]); }
	__device__ double tet(int a, int b, int c, int d) const { return f(a, b) * f(a, c) * f(a, d); }
	__device__ double tetOut(int a, int b, int c, int d) const { return (1 - f(a, b)) * (1 - f(a, c)) * (1 - f(a, d)); }
	__device__ double prism(int a0, int a1, int a2, int a3, int a4, int a5) const {
		const double e1 = f(a3, a4);
		return (f(a0, a1) + e1) * f(a1, a2) + e1 * f(a4, a5);
	}
	// crossing point of edge e, measured from its inside end
	__device__ void point(int e, double *p) const {
		const int a = c_edge[e][0], b = c_edge[e][1];
		const double fr = insideFrac(v[a], v[b]);
		const double t = v[a] < 0 ? fr : 1.0 - fr;
		const double pa[3] = {cornerX(a), cornerY(a), cornerZ(a)}, pb[3] = {cornerX(b), cornerY(b), cornerZ(b)};
#pragma unroll
		for (int k = 0; k < 3; k++) p[k] = pa[k] + t * (pb[k] - pa[k]);
	}
};
__device__ __forceinline__ double faceCut(double s, double t) { return (1 - 0.5 * (1 - s) * (1 - t)) / 3; }

// Closed form of canonical case `kase` (+32: case 9's second triangulation) on rotated values.
__device__ double canonicalVolume(int kase, const Cube &q) {
	const double k = 1.0 / 6.0;
	double P0[3], P1[3], P2[3], P3[3], P4[3], P5[3], P6[3];
	switch (kase) {
	case 0: return 0.0;
	case 1: return k * q.tet(0, 1, 3, 4);
	case 2: return k * q.prism(3, 0, 4, 2, 1, 5);
	case 3: return k * (q.tet(0, 1, 3, 4) + q.tet(5, 1, 6, 4));
	case 4: return k * (q.tet(0, 1, 3, 4) + q.tet(6, 7, 5, 2));
	case 5: {
		const double e3 = q.f(0, 3), e11 = q.f(3, 7);
		return q.f(1, 5) * (1 - 0.5 * (1 - q.f(0, 1)) * (1 - e3)) / 3 + k * ((q.f(2, 6) + e11) + e3 * e11);
	}
	case 6: return k * (q.prism(3, 0, 4, 2, 1, 5) + q.tet(6, 7, 5, 2));
	case 7: return k * (q.tet(4, 0, 5, 7) + q.tet(1, 0, 2, 5) + q.tet(6, 7, 5, 2));
	case 8: return k * (2 * q.f(0, 4) + q.f(1, 5) + 2 * q.f(2, 6) + q.f(3, 7));
	case 9:
	case 41: {  // points on edges 0, 1, 6, 7, 8, 10
		q.point(0, P0); q.point(1, P1); q.point(6, P2); q.point(7, P3); q.point(8, P4); q.point(10, P5);
		const double e10 = q.f(2, 6), e6 = q.f(6, 7);
		const double base = faceCut(e6, e10) + k * q.f(1, 2) * e10 + k * (e6 * q.f(4, 7));
		if (kase == 9) return base + k * (sv(P5, P3, P2) + sv(P1, P3, P5) + sv(P1, P4, P3) + sv(P1, P0, P4));
		return base + k * (sv(P5, P1, P0) + sv(P2, P5, P0) + sv(P2, P0, P4) + sv(P2, P4, P3));
	}
	case 10: return k * (q.prism(4, 7, 6, 0, 3, 2) + q.prism(2, 1, 0, 6, 5, 4));
	case 11: {  // points on edges 0, 1, 5, 6, 8, 11
		q.point(0, P0); q.point(1, P1); q.point(5, P2); q.point(6, P3); q.point(8, P4); q.point(11, P5);
		const double e5 = q.f(5, 6), e6 = q.f(6, 7);
		const double base = k * (q.f(1, 2) + e5) + faceCut(e6, q.f(3, 7)) + k * (e5 * e6);
		return base + k * (sv(P0, P4, P5) + sv(P0, P5, P2) + sv(P0, P2, P1) + sv(P2, P5, P3));
	}
	case 12: {
		const double e0 = q.f(0, 1), e9 = q.f(1, 5);
		return q.f(3, 7) * (1 - 0.5 * (1 - e0) * (1 - q.f(0, 3))) / 3 + k * ((e9 + q.f(2, 6)) + e0 * e9 + q.tet(4, 0, 5, 7));
	}
	case 13: return k * (q.tet(4, 0, 5, 7) + q.tet(1, 0, 2, 5) + q.tet(6, 7, 5, 2) + q.tet(3, 0, 2, 7));
	case 14: {  // points on edges 0, 3, 6, 7, 9, 10
		q.point(0, P0); q.point(3, P1); q.point(6, P2); q.point(7, P3); q.point(9, P4); q.point(10, P5);
		const double e10 = q.f(2, 6), e6 = q.f(6, 7);
		const double base = k * (q.f(1, 5) + e10) + k * (e6 * q.f(4, 7)) + faceCut(e6, e10);
		return base + k * (sv(P0, P1, P3) + sv(P0, P3, P5) + sv(P0, P5, P4) + sv(P2, P5, P3));
	}
	case 15: {  // points on edges 0, 1, 6, 7, 8, 10
		q.point(0, P0); q.point(1, P1); q.point(6, P2); q.point(7, P3); q.point(8, P4); q.point(10, P5);
		const double e10 = q.f(2, 6), e6 = q.f(6, 7);
		return faceCut(e6, e10) + k * q.f(1, 2) * e10 + k * (e6 * q.f(4, 7)) +
		       k * (sv(P1, P2, P5) + sv(P1, P3, P2) + sv(P1, P0, P3) + sv(P4, P3, P0)) + k * q.tet(5, 4, 1, 6);
	}
	case 16: {  // points on edges 1, 3, 5, 6, 8, 9, 10
		q.point(1, P0); q.point(3, P1); q.point(5, P2); q.point(6, P3); q.point(8, P4); q.point(9, P5); q.point(10, P6);
		const double e10 = q.f(2, 6), e5 = q.f(5, 6), e6 = q.f(6, 7);
		return k * (sv(P0, P1, P3) + sv(P0, P3, P6) + sv(P1, P4, P3) + sv(P2, P3, P5) + sv(P4, P5, P3)) +
		       k * (q.f(1, 2) * e10 + e5 * q.f(1, 5)) + faceCut(e6, e10) + faceCut(e6, e5);
	}
	case 17: {
		const double e3 = q.f(0, 3), e11 = q.f(3, 7);
		return 1 - ((1 - q.f(1, 5)) * (1 - 0.5 * q.f(0, 1) * e3) / 3 + k * ((1 - q.f(2, 6)) + (1 - e11) + (1 - e3) * (1 - e11)));
	}
	case 18: return 1 - k * (q.tetOut(0, 1, 3, 4) + q.tetOut(6, 5, 2, 7));
	case 19: {  // points on edges 0, 3, 4, 5, 8, 9
		q.point(0, P0); q.point(3, P1); q.point(4, P2); q.point(5, P3); q.point(8, P4); q.point(9, P5);
		const double e5 = q.f(5, 6);
		return 1 - (k * (-sv(P4, P2, P3) - sv(P4, P3, P1) - sv(P5, P0, P3) - sv(P0, P1, P3)) +
		            (0.5 * (1 - q.f(1, 5)) * (1 - e5)) / 3 + (0.5 * (1 - e5) * (1 - q.f(4, 5))) / 3);
	}
	case 20: {
		const double e1 = q.f(1, 2);
		return 1 - k * (((1 - q.f(0, 3)) + (1 - e1)) * (1 - q.f(0, 4)) + (1 - e1) * (1 - q.f(1, 5)));
	}
	case 21: return 1 - k * q.tetOut(0, 1, 3, 4);
	case 22: return 1.0;
	}
	return 0.0;
}

// Filled marching-squares area of one square (value <= 0 inside; a diagonal pair joins
// through the centre when the mean of the four values is <= 0: Contourer.cpp:86-93).
// c: (0,0), (1,0), (0,1), (1,1).
__device__ double squareArea(const double *c) {
	const double x[4] = {0, 1, 1, 0}, y[4] = {0, 0, 1, 1};
	const double v[4] = {c[0], c[1], c[3], c[2]};
	bool in[4];
	int nIn = 0;
#pragma unroll
	for (int i = 0; i < 4; i++) { in[i] = v[i] <= 0; nIn += in[i]; }
	if (nIn == 0) return 0.0;
	if (nIn == 4) return 1.0;
	if (nIn == 2 && in[0] == in[2] && !((c[0] + c[1] + c[2] + c[3]) / 4 <= 0)) {
		double area = 0;
		for (int i = 0; i < 4; i++) {
			if (!in[i]) continue;
			const int j = (i + 1) & 3, h = (i + 3) & 3;
			const double t1 = v[i] / (v[i] - v[j]), t2 = v[h] / (v[h] - v[i]);
			const double ax = (1 - t1) * x[i] + t1 * x[j], ay = (1 - t1) * y[i] + t1 * y[j];
			const double bx = (1 - t2) * x[h] + t2 * x[i], by = (1 - t2) * y[h] + t2 * y[i];
			area += 0.5 * fabs((ax - x[i]) * (by - y[i]) - (ay - y[i]) * (bx - x[i]));
		}
		return area;
	}
	double px[8], py[8];
	int n = 0;
	for (int i = 0; i < 4; i++) {
		const int j = (i + 1) & 3;
		if (in[i]) { px[n] = x[i]; py[n] = y[i]; n++; }
		if (in[i] != in[j]) {
			const double t = v[i] / (v[i] - v[j]);
			px[n] = (1 - t) * x[i] + t * x[j]; py[n] = (1 - t) * y[i] + t * y[j]; n++;
		}
	}
	double s = 0;
	for (int m = 0; m < n; m++) { const int l = (m + 1 == n) ? 0 : m + 1; s += px[m] * py[l] - px[l] * py[m]; }
	return 0.5 * s;
}

// Sum over the cubes (squares) between samples, per block; then one fixed-order sum.
template <int D, typename T>
__global__ void __launch_bounds__(kBlock) kVolumeCells(int sx, int sy, int sz, const T *__restrict__ f, int evaluatorOrder, double *partials) {
	__shared__ double sh[32];
	const int64_t nc = int64_t(sx - 1) * (sy - 1) * (D == 3 ? sz - 1 : 1);
	double acc = 0;
	for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < nc; c += int64_t(gridDim.x) * blockDim.x) {
		const unsigned u = unsigned(c), cx = unsigned(sx - 1), cy = unsigned(sy - 1);
		const unsigned r = u / cx, i = u - r * cx;
		const unsigned j = D == 3 ? r % cy : r, kk = D == 3 ? r / cy : 0;
		const int64_t base = int64_t(i) + int64_t(sx) * (int64_t(j) + int64_t(sy) * kk);
		const int64_t ox = 1, oy = sx, oz = int64_t(sx) * sy;
		if (D == 2) {
			const double s4[4] = {double(f[base]), double(f[base + ox]), double(f[base + oy]), double(f[base + ox + oy])};
			acc += squareArea(s4);
		} else {
			// the reference's stencil order, x fastest (GridBasedData.h:79-97)
			double s8[8] = {double(f[base]), double(f[base + ox]), double(f[base + oy]), double(f[base + ox + oy]),
			                double(f[base + oz]), double(f[base + ox + oz]), double(f[base + oy + oz]), double(f[base + ox + oy + oz])};
			if (evaluatorOrder) { double t = s8[2]; s8[2] = s8[3]; s8[3] = t; t = s8[6]; s8[6] = s8[7]; s8[7] = t; }
			int p = 0;
#pragma unroll
			for (int q = 0; q < 8; q++) p |= (s8[q] < 0 ? 1 : 0) << q;
			if (p == 0) continue;
			if (p == 255) { acc += 1.0; continue; }
			Cube cube;
#pragma unroll
			for (int q = 0; q < 8; q++) cube.v[q] = s8[c_mc.perm[p][q]];
			acc += canonicalVolume(c_mc.kase[p], cube);
		}
	}
	const double b = blockSum(acc, sh);
	if (threadIdx.x == 0) partials[blockIdx.x] = b;
}

// Fixed-order sum of the block sums; to `out`, or to the current step record.
__global__ void kVolumeTotal(const double *partials, int n, double scale, double *out, double *stats, const unsigned long long *counter) {
	if (threadIdx.x != 0 || blockIdx.x != 0) return;
	double s = 0;
	for (int b = 0; b < n; b++) s += partials[b];
	if (out) *out = s * scale;
	if (stats) {
		double *rec = stepRecord(stats, counter);
		if (rec) rec[kStVolume] = s * scale;
	}
}

// Enqueue the volume of tmp; the result goes to devOut and/or the current step record.
template <int D, typename T>
garm_status enqueueVolume(State &s, int evaluatorOrder, double *devOut, bool toRecord) {
	const int sx = s.geom.n[0], sy = s.geom.n[1], sz = D == 3 ? s.geom.n[2] : 1;
	const int64_t nc = int64_t(sx - 1) * (sy - 1) * (D == 3 ? sz - 1 : 1);
	const int cap = s.maxBlocks * 4;  // the partials buffer holds maxBlocks * 4 doubles
	const int blocks = int(std::max<int64_t>(1, std::min<int64_t>((nc + kBlock - 1) / kBlock, cap)));
	const double dx = s.geom.dx;
	kVolumeCells<D, T><<<blocks, kBlock, 0, s.stream>>>(sx, sy, sz, (const T *)s.tmp, evaluatorOrder, s.partials); s.launches++;
	kVolumeTotal<<<1, 32, 0, s.stream>>>(s.partials, blocks, D == 3 ? dx * dx * dx : dx * dx, devOut,
	                                      toRecord ? s.statsDev : nullptr, s.stepCounter); s.launches++;
	GARM_CHECK_LAUNCH();
	return GARM_OK;
}

}  // namespace

garm_status loadVolumeTables() { return ensureTables(); }

template <int D, typename T>
garm_status levelSetVolume(State &s, int evaluatorOrder, double *out) {
	if (D == 3) GARM_TRY(ensureTables());
	GARM_TRY((enqueueVolume<D, T>(s, evaluatorOrder, s.volumeOut, false)));
	if (cudaMemcpyAsync(out, s.volumeOut, sizeof(double), cudaMemcpyDeviceToHost, s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	if (cudaStreamSynchronize(s.stream) != cudaSuccess) return GARM_CUDA_ERROR;
	return GARM_OK;
}

template <int D, typename T>
garm_status recordVolumeAsync(State &s) {
	return enqueueVolume<D, T>(s, 0, nullptr, true);  // tables are loaded at creation
}

#define GARM_INST(D, T) template garm_status levelSetVolume<D, T>(State &, int, double *); template garm_status recordVolumeAsync<D, T>(State &);
GARM_INST(2, double)
GARM_INST(3, double)
GARM_INST(2, float)
GARM_INST(3, float)
#undef GARM_INST

}  // namespace garm
