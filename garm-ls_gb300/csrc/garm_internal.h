// garm_internal.h — device state of one simulation and the stage entry points
// shared by the kernel translation units and the C ABI (garm_capi.cu).
#pragma once

#include "../../include/garm.h"
#include "garm_device.cuh"

#include <cstddef>
#include <cstdint>
#include <utility>
#include <cuda_runtime.h>

namespace garm {

// Device buffers of one LevelSetLiquid<Dim> (Source/Core/LevelSetLiquid.h:27-121).
// Field planes are stored in the working type T of the precision mode:
// double for GARM_PRECISION_FP64, float for GARM_PRECISION_MIXED.
struct State {
	Geom geom{};
	garm_config cfg{};
	int dim = 3;
	bool mixed = false;
	size_t esz = 8;            // bytes per stored field element
	cudaStream_t stream = nullptr;
	bool ownStream = false;
	// a second stream for independent stages: forked from and joined back to `stream` by
	// events, so a captured step has them as parallel branches
	cudaStream_t aux = nullptr;
	cudaEvent_t forkEv[2] = {}, joinEv[2] = {};
	int numSMs = 0;
	long long stepIndex = 0;
	long long launches = 0;    // kernels launched by this simulation (for the bench's gpu_launches)

	int64_t N = 0, NN = 0;     // cells, nodes
	int64_t F[3] = {0, 0, 0};  // faces per axis
	int64_t Ftot = 0;

	// velocity (_velocity) and advection ping-pong
	void *u[3] = {}, *uNew[3] = {};
	void *uGrad[9] = {};       // [axis*3+b]: d u_axis / d x_b on face grid `axis` (Derivatives::computeFirst<2>)
	// reference map ξ and Jacobian Π (planes col*D+row)
	void *xi[3] = {}, *xiNew[3] = {};
	void *Pi[9] = {}, *PiNew[9] = {};
	void *xiMixed[12] = {};    // Hermite mixed derivatives of ξ: [m*3+comp]
	// level sets
	void *phi = nullptr, *tmp = nullptr, *ori = nullptr, *ref = nullptr;
	void *refGrad[3] = {};     // ψ0 = ∇φ0 (_refLevelSetGrad)
	void *refMixed[4] = {};    // cached Hermite mixed derivatives of φ0 (_refLevelSetView)
	void *rA = nullptr, *rB = nullptr;  // reinitialisation RK stages
	// Newton configuration only (cfg.restart_newton): ∇φ of the composed level set
	// (_levelSetGrad) and the HybridNewton work buffers
	void *lsGrad[3] = {};
	void *hnPhi = nullptr, *hnGrad[3] = {}, *hnMixed[4] = {}, *hnPoints[3] = {};
	uint8_t *hnMark[2] = {};
	// fast-marching configuration only (cfg.fast_marching): tentative distances, seed
	// flags, the relaxation's barrier and control words
	void *marchTent = nullptr, *marchTent2 = nullptr;
	uint8_t *marchFixed = nullptr;
	int *marchStamp = nullptr;         // per cell: the last relaxation sweep it was queued for
	unsigned *marchBar = nullptr;
	int *marchInts = nullptr;
	uint8_t *adv = nullptr;    // _advRegion
	uint8_t *vis0 = nullptr;   // cell extrapolation levels (seed 0, joined in pass p, 255 unreached)
	uint8_t *fvis0 = nullptr;  // face extrapolation levels (all axes, concatenated)
	// frontier extrapolation: queued-once bits, the two frontier lists, per-pass sizes; a
	// second set for the face march, which runs beside the cell marches
	unsigned *frontBits = nullptr, *frontBitsB = nullptr;
	int *frontList[2] = {}, *frontListB[2] = {};
	int *frontCount = nullptr, *frontCountB = nullptr;
	// boundary (Boundary<Dim>, Source/Core/Boundary.h:16-24)
	void *cellDist = nullptr, *nodeDist = nullptr;
	void *fraction[3] = {}, *bvel[3] = {}, *normal[3] = {};
	int64_t *bcList = nullptr; int64_t nBc = 0;   // faces with fraction > 0.1 (Boundary::enforce work list), concatenated face ids
	void *bcTmp = nullptr;
	// projection (Projector<Dim>, Source/Core/Projector.h:14-21)
	int *grid2mat = nullptr;   // cell -> unknown id or -1
	int *mat2grid = nullptr;   // unknown id -> cell
	int *scanBlock = nullptr;  // per-block counts for the compaction scan
	int *nUnknownsDev = nullptr;
	int nUnknowns = 0;
	void *ent64 = nullptr;      // [2D][N] {neighbour unknown id (-1: none), weight w}, matrix entry -w (FP64)
	void *ent32 = nullptr;      // the same entries with FP32 weights (mixed)
	unsigned *rowHdr = nullptr; // compact rows of the streamed solves: [N] presence bits, full-row flag, y distances
	int *rowIdx = nullptr;      // [N][2] neighbour ids of the z entries (3D)
	double *diag = nullptr, *invd = nullptr, *rhs = nullptr, *pres = nullptr;
	float *diag32 = nullptr, *invd32 = nullptr;
	// PCG work vectors: packed {r, w, s, 1/diag} per unknown (double-buffered, in the
	// solve's element type), the search direction, the mixed form's FP32 correction
	// and its FP64 refinement residual cgR
	double *cgR = nullptr;
	void *cgPack[2] = {};
	double *cgP64 = nullptr;
	float *cgP32 = nullptr, *cgE32 = nullptr;
	double *partials = nullptr; int maxBlocks = 0;
	double *volumeOut = nullptr;   // result slot of the volume diagnostic
	unsigned *barrier = nullptr;   // [count, generation]
	double *cgScalars = nullptr;   // device-side scalars written by the persistent solver
	int *cgInts = nullptr;
	// reductions
	unsigned long long *redU64 = nullptr;
	int *redI32 = nullptr;  // 16 ints: reduction counts; [kRestartOverride] the restart override
	// device staging for AoS<->SoA transfers
	void *stage = nullptr; size_t stageBytes = 0;
	// every device allocation, freed by garm_sim_destroy
	void *allocs[160] = {}; int nAllocs = 0; size_t deviceBytes = 0;
	bool dryRun = false;       // count allocation sizes only (garm_sim_estimate_bytes)
	// timing events
	cudaEvent_t ev[10] = {};
	// device-resident stepping: dt of the current step, the Simulator frame clock
	// {time in frame, frame length, cfl}, the restart decision (gates the restart
	// branch when non-null) and per-step statistics written on the device
	double *dtDev = nullptr;
	double *clockDev = nullptr;
	int *restartFlag = nullptr;
	const int *gate = nullptr;
	int *reinitErr = nullptr;          // set by a tiled reinitialisation whose staged plane did not arrive
	bool inStep = false;               // enqueueing a step: stage errors go to its device record
	double *statsDev = nullptr;        // kStatsSlots doubles per recorded step
	unsigned long long *stepCounter = nullptr;  // device count of started steps
	unsigned long long hostSteps = 0;           // host mirror of the counter
	double *statsHost = nullptr;       // pinned mirror
	int statsCap = 0;
	// captured single-step graphs (even / odd step: the ping-pong buffers alternate)
	cudaGraphExec_t stepGraph[2] = {nullptr, nullptr};
	bool graphTried = false, graphOk = false;
	void *evenU0 = nullptr;            // u[0] buffer of the even-step graph
	long long graphLaunches = 0;       // kernels in one captured step
	int pendingSteps = 0;              // steps enqueued and not yet collected
};

// Per-step records live in a device ring indexed by a device step counter, so a
// captured step graph writes the record of whichever step it is replaying.
constexpr int kStatsCap = 256;
__device__ __forceinline__ double *stepRecord(double *base, const unsigned long long *counter) {
	return base ? base + ((*counter + kStatsCap - 1) % kStatsCap) * 12 : nullptr;
}

// Layout of one per-step statistics record on the device.
enum StatSlot { kStDt = 0, kStRestarted, kStRmTotal, kStRmBad, kStUnknowns, kStCgIters, kStCgRefine, kStCgResidual, kStCgTol, kStCgErr, kStVolume, kStPersistErr, kStatsSlots = 12 };

// Stage entry points (templated on dimension D and working type T).
template <int D, typename T> garm_status initBoundary(State &s);
template <int D, typename T> garm_status finishBoundary(State &s);
template <int D, typename T> garm_status advectFields(State &s);
template <int D, typename T> garm_status generateCurrentFields(State &s);
template <int D, typename T> garm_status reinitialize(State &s);
// calculateVolume of tmp (synchronises the stream); evaluatorOrder: 3D corner order (see garm.h).
template <int D, typename T> garm_status levelSetVolume(State &s, int evaluatorOrder, double *out);
// The same enqueued on the stream with the result written to the current step record.
template <int D, typename T> garm_status recordVolumeAsync(State &s);
// Load the volume tables onto the current device (before any stream capture).
garm_status loadVolumeTables();
// Launch plan (form GARM_REINIT_*, threads per block, cells per thread) the
// reinitialisation autotuner chose for this grid, and its sub-stage time in ms.
template <int D, typename T> garm_status reinitPlanInfo(State &s, int *form, int *block, int *chunk, float *ms);
garm_status pinReinitPlan(int dim, int esz, const int *size, int form, int block, int chunk);
// GARM_TIMEOUT once a TMA-staged plane of the tiled reinitialisation form did not arrive
// within its bounded wait (sticky); synchronises the stream.
garm_status tiledReinitStatus(cudaStream_t st, const int *err);
template <int D, typename T> garm_status extrapolateToCollider(State &s);
template <int D, typename T> garm_status checkReferenceMap(State &s, int *keep, int *tot, int *bad);
template <int D, typename T> garm_status checkReferenceMapAsync(State &s, bool record);
template <int D, typename T> garm_status restart(State &s);
template <int D, typename T> garm_status bodyForce(State &s);
template <int D, typename T> garm_status project(State &s, garm_step_stats *st);
template <int D, typename T> garm_status projectAsync(State &s, bool record);
garm_status projectStats(State &s, garm_step_stats *st);
garm_status pcgPrepare();
template <int D, typename T> garm_status extrapolateToAir(State &s);
constexpr int kFrontMaxPasses = 250;  // extrapolation passes fit a level byte (255 = unreached)
template <int D, typename T> garm_status enforceBoundaryConditions(State &s);
template <int D, typename T> garm_status enforceBoundaryLevelSet(State &s, void *field, double tol);
template <int D, typename T> garm_status resetRefView(State &s);
// Hermite mixed derivatives of a scalar field from its gradient planes (gated by s.gate).
template <int D, typename T> garm_status scalarMixed(State &s, T *const *grad, T *const *mixed);
template <int D, typename T> garm_status initRefMap(State &s);
template <int D, typename T> garm_status refreshRefGradient(State &s);
template <int D, typename T> garm_status levelSetGradient(State &s);
// FastMarching::perform on a cell plane: seeds from the sign changes of φ (mark null) or
// the marked cells, then the relaxation and the sign; errors go to the step record when
// `record` is set, else marchStatus reads them.
template <int D, typename T> garm_status fastMarch(State &s, void *phi, const uint8_t *mark, int maxSteps, bool record);
garm_status marchStatus(State &s, int *sweeps);
template <int D, typename T> garm_status maxSpeed(State &s, double *out);
template <int D, typename T> garm_status maxSpeedAsync(State &s);
// Zeroes the first na words of a and nb words of b (one block of 32 threads).  Steps clear
// their counters with this kernel, not with memset nodes: memset nodes of concurrently
// replayed step graphs serialise against each other.
__global__ void kClearWords(unsigned *a, int na, unsigned *b, int nb);
__global__ void kStepDt(const unsigned long long *maxBits, double dx, double *clock, double *dt, double *stats, const unsigned long long *counter);
template <int D, typename T> garm_status copyField(State &s, void *dst, const void *src, int64_t n);

// Standalone WENO5 reinitialisation on raw device planes.  With tune = false a shape
// that has no cached or pinned launch plan runs the default column plan instead of
// timing the candidates (no event creation, no stream synchronisation).
template <int D, typename T> garm_status reinitRaw(cudaStream_t st, const int *size, double dx, T *phi, T *a, T *b, int iters, double cfl, int *err, bool tune = true);

constexpr int kRestartOverride = 8;  // word of State::redI32 that garm_sim_set_restart_override sets

inline garm_status cudaStatus(cudaError_t e) { return e == cudaSuccess ? GARM_OK : GARM_CUDA_ERROR; }
// Work after forkAux(k) on s.aux runs beside work on s.stream until joinAux(k).
inline garm_status forkAux(State &s, int k) {
	if (cudaEventRecord(s.forkEv[k], s.stream) != cudaSuccess || cudaStreamWaitEvent(s.aux, s.forkEv[k], 0) != cudaSuccess) return GARM_CUDA_ERROR;
	return GARM_OK;
}
inline garm_status joinAux(State &s, int k) {
	if (cudaEventRecord(s.joinEv[k], s.aux) != cudaSuccess || cudaStreamWaitEvent(s.stream, s.joinEv[k], 0) != cudaSuccess) return GARM_CUDA_ERROR;
	return GARM_OK;
}
#define GARM_CHECK_LAUNCH() do { cudaError_t _e = cudaGetLastError(); if (_e != cudaSuccess) return GARM_CUDA_ERROR; } while (0)
#define GARM_TRY(x) do { garm_status _s = (x); if (_s != GARM_OK) return _s; } while (0)

inline unsigned gridFor(int64_t n, int block = kBlock) { return unsigned((n + block - 1) / block); }

// Launch with programmatic stream serialisation: the kernel (which calls pdlWait() before
// touching global memory) is scheduled during the previous kernel's tail instead of after it.
template <typename... K, typename... A>
inline cudaError_t launchPdl(void (*kernel)(K...), dim3 grid, dim3 block, cudaStream_t st, A &&...args) {
	cudaLaunchConfig_t cfg = {};
	cfg.gridDim = grid;
	cfg.blockDim = block;
	cfg.dynamicSmemBytes = 0;
	cfg.stream = st;
	cudaLaunchAttribute at[1];
	at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
	at[0].val.programmaticStreamSerializationAllowed = 1;
	cfg.attrs = at;
	cfg.numAttrs = 1;
	return cudaLaunchKernelEx(&cfg, kernel, std::forward<A>(args)...);
}

}  // namespace garm
