/*
 * garm.h — C ABI of the GB300 per-timestep GARM-LS grid pipeline.
 *
 * One opaque simulation handle owns the device state of one liquid scene on one
 * GPU.  Every call returns a garm_status; nothing exits the process.  Host
 * buffers passed to upload/download use the byte layout of the reference's
 * frame files (`*.sav`): raw native-endian arrays written by
 * GridBasedData::save (Source/Core/GridBasedData.h:102-103, Common/Util/IO.h:20-26),
 * x-fastest cell order (Source/Core/Grid.h:40-44), vector fields interleaved
 * per cell, matrices column-major per cell (Common/Util/Types.h:52-54), and the
 * D face arrays of a staggered field in axis order (Source/Core/SGridBasedData.h:54-55).
 *
 * The entry points replace the stage methods of
 * LevelSetLiquid<Dim> (Source/Core/LevelSetLiquid.h:125-169); the host C++
 * class in garm-ls_gb300/host/GpuLevelSetLiquid.h wraps them behind the
 * reference's Simulation interface (Common/Util/Simulation.h:10-34).
 */
#ifndef GARM_H
#define GARM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GARM_ABI_VERSION 5

typedef enum garm_status {
    GARM_OK = 0,
    GARM_INVALID = 1,        /* bad argument, size or field id */
    GARM_OOM = 2,            /* device allocation failed */
    GARM_NOT_CONVERGED = 3,  /* pressure PCG hit its iteration cap (reference: LinearSystem.h:33-36 exits) */
    GARM_NUMERIC = 4,        /* NaN/Inf found in an input or in the state */
    GARM_CUDA_ERROR = 5,     /* a CUDA runtime call failed */
    GARM_TIMEOUT = 6,        /* a bounded device-side wait gave up (grid barrier, or a TMA-staged
                                plane of the tiled reinitialisation form); the fields the call was
                                writing are not usable: reload or recreate the simulation */
    GARM_UNSUPPORTED = 7     /* feature not built into this library */
} garm_status;

typedef enum garm_precision {
    GARM_PRECISION_FP64 = 0,  /* plain form: every stage in FP64, as the reference */
    GARM_PRECISION_MIXED = 1  /* FP32 storage+math for advection/Hermite/WENO/matvec; FP64-class dot
                                 products, FP64 true residuals (residual replacement) and the
                                 reference-map test in FP64 */
} garm_precision;

/* Field ids for upload/download.  Byte sizes follow the reference's .sav layout. */
typedef enum garm_field {
    GARM_FIELD_VELOCITY = 0,            /* D face arrays of double (LevelSetLiquid::_velocity)           */
    GARM_FIELD_LEVEL_SET = 1,           /* cell double   (_levelSet)                                     */
    GARM_FIELD_REF_MAP = 2,             /* cell double[D] (_refMap, refMap.sav)                          */
    GARM_FIELD_REF_MAP_GRAD = 3,        /* cell double[D*D] column-major (_refMapGrad, refMapGrad.sav)   */
    GARM_FIELD_REF_LEVEL_SET = 4,       /* cell double   (_refLevelSet, refLevelSet.sav)                 */
    GARM_FIELD_REF_LEVEL_SET_GRAD = 5,  /* cell double[D] (_refLevelSetGrad)                             */
    GARM_FIELD_ADV_REGION = 6,          /* cell uint8    (_advRegion, advRegion.sav)                     */
    GARM_FIELD_ORI_LEVEL_SET = 7,       /* cell double   (_oriLevelSet)                                  */
    GARM_FIELD_TMP_LEVEL_SET = 8,       /* cell double   (_tmpLevelSet)                                  */
    GARM_FIELD_CELL_DIST = 9,           /* cell double   (Boundary::cellDist)                            */
    GARM_FIELD_NODE_DIST = 10,          /* node double   (Boundary::nodeDist)                            */
    GARM_FIELD_FRACTION = 11,           /* D face arrays (Boundary::fraction)                            */
    GARM_FIELD_BOUNDARY_VELOCITY = 12,  /* D face arrays (Boundary::velocity)                            */
    GARM_FIELD_BOUNDARY_NORMAL = 13,    /* D face arrays (Boundary::normal)                              */
    GARM_FIELD_PRESSURE = 14,           /* cell double: last solved pressure, 0 off the unknown set      */
    GARM_FIELD_LEVEL_SET_GRAD = 15,     /* cell double[D] (_levelSetGrad; restart_newton only)           */
    GARM_FIELD_COUNT = 16
} garm_field;

/* StaggeredGrid(boundaryWidth, spacing, resolution, center)
 * (Source/Core/StaggeredGrid.h:27-36).  resolution counts cells including the
 * solid ring; unused components of 2D grids are ignored. */
typedef struct garm_grid_desc {
    int dim;                 /* 2 or 3 */
    int resolution[3];
    int boundary_width;      /* 2 in every reference scene */
    double spacing;          /* dx */
    double center[3];
} garm_grid_desc;

/* Runtime knobs.  Defaults (garm_config_default) equal the reference constants. */
typedef struct garm_config {
    int precision;                    /* garm_precision */
    int reinit_iters;                 /* 30   (LevelSetLiquid.cpp:1156) */
    double reinit_cfl;                /* 0.9  (LevelSetLiquid.cpp:1156) */
    int reinit_interval;              /* 1: reinitialise every step (LevelSetLiquid.cpp:625) */
    double cg_tolerance;              /* 1e-8 relative residual (Jacobi-PCG; the reference's Eigen IC-PCG uses 1e-5) */
    int cg_max_iters;                 /* 2000 (Projector.cpp:161) */
    double boundary_extrap_radius;    /* 6    (LevelSetLiquid.h:92)  */
    double air_extrap_radius;         /* 15   (LevelSetLiquid.h:93)  */
    double rm_threshold;              /* 0.883022221559489 (LevelSetLiquid.cpp:631) */
    double rm_band;                   /* 4   */
    double rm_ratio;                  /* 1e-5 */
    int enable_gravity;               /* 1   (LevelSetLiquid.h:72) */
    double mixed_residual_drop;       /* mixed only: the FP32 PCG's residual is replaced by the FP64 true
                                         residual b - A x each time it has dropped by this factor */
    int mixed_replace_interval;       /* mixed only: replace at least every this many iterations (0: never
                                         by count) */
    int cg_cells_per_block;           /* pressure solve: one 512-thread block (one SM) per this many interior
                                         cells, at most one per SM; 0 selects 4096.  Larger values leave
                                         SMs free for other scenes' work when scenes run concurrently */
    int record_volume;                /* 1: every step ends with the volume diagnostic (garm_sim_volume, corner
                                         order 0) written to its statistics on the device (no host round trip) */
    int restart_newton;               /* 1: the reference's Newton configuration (_ENABLE_NEWTON_):
                                         compose also keeps ∇φ = Πᵀ∇φ₀(ξ), initialize takes ψ₀ from the 4th-order
                                         gradient of φ, and restart() is the HybridNewton closest-point restart
                                         (LevelSetLiquid.cpp:1290-1308); 0: the plain restart */
    int fast_marching;                /* 1: the reference's fast-marching configuration (_ENABLE_FMM_):
                                         reinitializeLevelSet is fast marching over a band of 15 cells
                                         (LevelSetLiquid.cpp:1151-1152) instead of WENO5, and the Newton
                                         restart ends with a fast-marching sweep (HybridNewton.cpp:51-64)
                                         instead of eikonal advection.  Both flags set is the reference's
                                         default build (xmake.lua:41-55) */
} garm_config;

/* Per-step statistics returned by garm_sim_advance. */
typedef struct garm_step_stats {
    int restarted;            /* 1 when checkReferenceMap failed and restart() ran */
    int cg_iterations;        /* total PCG iterations (inner iterations summed in mixed mode) */
    int cg_refinements;       /* FP64 residual replacements (mixed); 1 in FP64 */
    int unknowns;             /* pressure unknowns of this step */
    double cg_residual;       /* final relative residual |b-Ax|/|b| */
    int rm_total;             /* band cells inspected by checkReferenceMap */
    int rm_bad;               /* band cells whose Jacobian columns are near-parallel */
    double ms_total;          /* device time of the step (CUDA events) */
    double ms_stage[8];       /* advect, compose, reinit, extrap_collider, rm_check+restart,
                                 body_force, project, extrap_air+enforce_bc */
    double volume;            /* liquid volume after the step when record_volume is set, else 0 */
} garm_step_stats;

typedef struct garm_sim garm_sim;

/* Library identity. */
int garm_abi_version(void);
const char *garm_status_string(garm_status s);
garm_status garm_config_default(garm_config *cfg);

/* Lifetime.  `stream` is a cudaStream_t (NULL: the library creates its own).
 * Replaces LevelSetLiquid<Dim>::LevelSetLiquid(const StaggeredGrid<Dim>&)
 * (Source/Core/LevelSetLiquid.cpp:46-77) plus Boundary::Boundary/reset
 * (Source/Core/Boundary.cpp:8-35) for the domain box walls. */
garm_status garm_sim_create(const garm_grid_desc *grid, const garm_config *cfg, void *stream, garm_sim **out);
garm_status garm_sim_destroy(garm_sim *sim);
/* Device bytes garm_sim_create would allocate for this grid and configuration,
 * without allocating (admission control; no reference counterpart).  A grid or a
 * configuration that garm_sim_create would refuse returns GARM_INVALID here too. */
garm_status garm_sim_estimate_bytes(const garm_grid_desc *grid, const garm_config *cfg, size_t *bytes);
garm_status garm_sim_device_bytes(const garm_sim *sim, size_t *bytes);
/* Kernels launched by this simulation since creation (no reference counterpart: instrumentation). */
garm_status garm_sim_launch_count(const garm_sim *sim, long long *count);

/* Host <-> device transfer in the .sav layout.  Replaces GridBasedData::save/load
 * (Source/Core/GridBasedData.h:102-103) as used by LevelSetLiquid::saveFrame/
 * loadFrame (Source/Core/LevelSetLiquid.cpp:425-526). */
garm_status garm_sim_field_bytes(const garm_sim *sim, int field, size_t *bytes);
garm_status garm_sim_upload(garm_sim *sim, int field, const void *host, size_t bytes);
garm_status garm_sim_download(garm_sim *sim, int field, void *host, size_t bytes);

/* LevelSetLiquid::initialize (Source/Core/LevelSetLiquid.cpp:528-598), RM+GA, FMM off;
 * the Newton branches when restart_newton is set.  Expects the velocity and level set
 * uploaded first. */
garm_status garm_sim_initialize(garm_sim *sim);

/* The non-I/O part of LevelSetLiquid::loadFrame (Source/Core/LevelSetLiquid.cpp:474-526),
 * to call after uploading velocity, refMap, refLevelSet, advRegion and refMapGrad (and, with
 * restart_newton, refLevelSetGrad): Boundary::finish, ψ0 = computeFirst<4>(φ0) unless
 * restart_newton is set, and the Hermite view reset. */
garm_status garm_sim_finish_load(garm_sim *sim);

/* LevelSetLiquid::advance (Source/Core/LevelSetLiquid.cpp:608-698). `stats` may be NULL. */
garm_status garm_sim_advance(garm_sim *sim, double dt, garm_step_stats *stats);

/* Device-resident stepping.  garm_sim_set_clock starts a frame clock for the
 * Simulator's dt policy (Common/Util/Simulator.cpp:102-128): dt = cfl*dx/max|u|,
 * clamped to the end of a frame of 1/frame_rate seconds and halved when two steps
 * remain.  garm_sim_advance_auto then runs `steps` advance() calls with dt computed
 * on the device, replaying a captured CUDA graph of one step when the device
 * allows it, and synchronises once at the end; `stats` describes the last step and
 * ms_total the whole call.  Replaces the Simulator loop around advance(). */
garm_status garm_sim_set_clock(garm_sim *sim, unsigned frame_rate, double cfl);
garm_status garm_sim_advance_auto(garm_sim *sim, int steps, garm_step_stats *stats);
/* Asynchronous form for serving loops: enqueue `steps` auto steps on the
 * simulation's stream and return at once; poll for completion; collect the
 * statistics (waits if needed).  Scenes on different streams overlap on the GPU. */
garm_status garm_sim_enqueue_auto(garm_sim *sim, int steps);
garm_status garm_sim_poll(garm_sim *sim, int *done);
garm_status garm_sim_collect(garm_sim *sim, garm_step_stats *stats);
/* Batched scenes: `steps` auto steps of every simulation, issued round-robin one
 * step per scene on each scene's own stream (create the simulations with a NULL
 * stream so each owns one).  stats (may be NULL) receives one record per scene.
 * A scene's results do not depend on the batch it runs in. */
garm_status garm_batch_advance_auto(garm_sim *const *sims, int count, int steps, garm_step_stats *stats);
/* Restart decision of the following steps (no reference counterpart): GARM_RESTART_AUTO is
 * checkReferenceMap's test (LevelSetLiquid.cpp:631); NEVER keeps the reference map and ALWAYS
 * restarts, whatever the test finds.  For experiments that hold one run's restart schedule
 * fixed in another, e.g. the mixed form on the FP64 form's schedule.  Applies from the next
 * step enqueued on the simulation's stream, captured step graphs included. */
#define GARM_RESTART_AUTO 0
#define GARM_RESTART_NEVER 1
#define GARM_RESTART_ALWAYS 2
garm_status garm_sim_set_restart_override(garm_sim *sim, int mode);
/* 1 when garm_sim_advance_auto replays captured step graphs (no reference counterpart). */
garm_status garm_sim_graph_active(const garm_sim *sim, int *active);
/* Launch forms of the WENO5 reinitialisation sub-stages (no reference counterpart):
 * one thread per cell; threads walking columns along the last axis; one pass
 * per axis, threads walking lines of that axis; (3D FP32) columns whose in-plane
 * stencils read tiles of each plane staged in shared memory by TMA, 128 threads per
 * block; or (3D FP32, rows of even length) threads walking two x-adjacent columns
 * as the two lanes of paired FP32 instructions, sharing the x face set between them;
 * or (3D FP32, rows of a multiple of 4 cells) that pair form with its in-plane stencils
 * read from TMA-staged plane tiles, 128 threads per block (other precisions and shapes
 * run the column form, or the pair form for even rows). */
#define GARM_REINIT_CELLS 0
#define GARM_REINIT_COLUMNS 1
#define GARM_REINIT_SWEEPS 2
#define GARM_REINIT_TILED 3
#define GARM_REINIT_PAIRS 4
#define GARM_REINIT_PAIRS_TILED 5
/* The launch plan the reinitialisation autotuner chose for this simulation's grid:
 * form, threads per block, cells each thread walks and the timed sub-stage in ms.
 * Plans are tuned once per grid shape, precision and device in the process, on
 * first use outside stream capture. */
garm_status garm_sim_reinit_plan(garm_sim *sim, int *form, int *threads, int *cells_per_thread, float *ms);
/* Pin the reinitialisation plan of one grid shape (cell counts per axis, storage
 * layout) and precision on the current device, replacing the autotuner's choice.
 * For every form but the cell form threads is 32..256 (a multiple of 32) and
 * cells_per_thread >= 1 (the cells, or planes, each thread walks); the cell form
 * ignores both, and the two tiled forms always run 128 threads per block.  threads 0
 * forgets the pinned or tuned plan, so the next use tunes again. */
garm_status garm_reinit_plan_set(int dim, int precision, const int *size, int form, int threads, int cells_per_thread);

/* calculateVolume (Source/Core/LevelSetLiquid.cpp:1162-1190): volume (2D: area) of the
 * liquid from the tmp level set, kept outside the timed step as a diagnostic.  2D sums the
 * filled marching-squares contour; 3D sums the marching-cubes-style volume of every cube
 * between samples (MC-style-vol-eval/fraction.hpp).  evaluator_order 0 passes each cube's
 * corners as the reference does (x-fastest stencil order, which swaps two corner pairs
 * relative to the evaluator's convention; first-order accurate); 1 passes them in the
 * evaluator's own order (second-order accurate; no reference counterpart). */
garm_status garm_sim_volume(garm_sim *sim, int evaluator_order, double *out);

/* max over faces of |u| (GridBasedData::normMax, Source/Core/GridBasedData.h:55-68). */
garm_status garm_sim_max_speed(garm_sim *sim, double *out);
/* LevelSetLiquid::getTimeStep (Source/Core/LevelSetLiquid.h:129): cfl*dx/max|u| (may be +inf). */
garm_status garm_sim_time_step(garm_sim *sim, double cfl, double *dt);

/* Single stages, for parity checks and for callers that drive the pipeline
 * themselves.  Each mirrors one protected method of LevelSetLiquid<Dim>. */
garm_status garm_stage_advect(garm_sim *sim, double dt);           /* advectFields       LevelSetLiquid.cpp:718-832  */
garm_status garm_stage_compose(garm_sim *sim);                     /* generateCurrentFields        :1218-1244       */
garm_status garm_stage_reinit(garm_sim *sim);                      /* reinitializeLevelSet         :1148-1160       */
garm_status garm_stage_extrap_collider(garm_sim *sim);             /* extrapolateFieldsToCollider  :1086-1137       */
garm_status garm_stage_rm_check(garm_sim *sim, int *keep, int *total, int *bad); /* checkReferenceMap :1246-1283 */
garm_status garm_stage_restart(garm_sim *sim);                     /* restart (plain branch)       :1285-1352       */
garm_status garm_stage_body_force(garm_sim *sim, double dt);       /* applyBodyForces              :834-877         */
garm_status garm_stage_project(garm_sim *sim, garm_step_stats *stats); /* projectVelocity         :1019-1023       */
garm_status garm_stage_extrap_air(garm_sim *sim);                  /* extrapolateFieldsToAir       :1059-1084       */
garm_status garm_stage_enforce_bc(garm_sim *sim);                  /* enforceBoundaryConditions    :1139-1146       */
garm_status garm_stage_enforce_boundary_level_set(garm_sim *sim, double tolerance); /* enforceBoundaryLevelSet :966-975 */

/* Standalone WENO5 reinitialisation of one cell field held on the host
 * (Reinitialization::solve<5>, Source/Core/Reinitialization.h:50-80), as the
 * reference's TestReinit program calls it (Source/Test/TestReinit/TestReinit.cpp:225-236).
 * `size` has `dim` entries; `phi` is updated in place. */
garm_status garm_reinit_host(int dim, const int *size, double spacing, double *phi, int iters, double cfl, int precision);

/* WENO5 reinitialisation of a cell field that is already in device memory, for
 * callers that may not allocate device memory: a plug-in whose host application
 * owns all GPU memory, or a real-time loop that cannot afford the implicit
 * synchronisation of cudaMalloc/cudaFree.  This entry point has no counterpart in
 * the reference; it runs the same kernels as garm_reinit_host.
 *
 * `phi` is a device pointer to size[0]*...*size[dim-1] doubles (x fastest),
 * updated in place on `stream` (a cudaStream_t; NULL = legacy default stream).
 * It calls no cudaMalloc, cudaFree or allocating library routine: its two stage
 * planes live in one fixed device array of 2*GARM_NOALLOC_MAX_CELLS doubles
 * (8 MiB), held by every GPU that loads the library until the process exits.
 * Grids of more than GARM_NOALLOC_MAX_CELLS cells return GARM_INVALID, and so does
 * a `phi` that is not memory of the current device or managed memory (a host
 * pointer, for instance).
 * The first call on a device looks up that array's device address
 * (cudaGetSymbolAddress, with that device current); make that first call before
 * any stream capture.  No call runs the reinitialisation autotuner or waits for
 * the stream: the launch plan is the one cached or pinned for the grid shape on
 * this device (garm_reinit_plan_set, or an earlier garm_reinit_host call of the
 * same shape), else the default column plan.  All calls share the one array, so
 * calls whose work overlaps on the GPU race; the array needs no clearing between
 * calls. */
#define GARM_NOALLOC_MAX_CELLS (1 << 19)
garm_status garm_reinit_device_noalloc(int dim, const int *size, double spacing, double *phi, int iters, double cfl, void *stream);

/* Self-test of the grid barrier that the persistent pressure solve and the fast-marching
 * relaxation use (no counterpart in the reference).  One cooperative launch of `blocks`
 * blocks passes `rounds` barriers in a row; *ms_per_barrier is the launch's device time
 * per barrier passed.  With never_complete = 1 the blocks wait for a count that is never
 * reached: every wait is bounded (about 2 s), and the call returns GARM_TIMEOUT with the
 * context still usable.  `blocks` above the co-resident limit returns GARM_INVALID. */
garm_status garm_barrier_selftest(int blocks, int rounds, int never_complete, double *ms_per_barrier);

/* FP64 FMA throughput of the current device (no counterpart in the reference): one launch
 * of blocks_per_sm × SMs blocks of 256 threads, each thread `iters` rounds of 8 independent
 * FMA chains, timed with CUDA events (shortest of three after one untimed launch).
 * *tflops counts an FMA as two operations.  It reads no clocks and changes none.  This is
 * the compute peak the plain FP64 form's stencil kernels are measured against. */
garm_status garm_fp64_peak_selftest(int blocks_per_sm, int iters, double *tflops);

#ifdef __cplusplus
}
#endif

#endif /* GARM_H */
