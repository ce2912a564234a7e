/*
 * analyticmesh_gb300.h -- C ABI of the GB300 Analytic Marching engine.
 *
 * The first five entry points are the reference's pybind11 module `cuam`
 * (backend/src/cuam.cpp:186-217, imported by backend/main.py:13) restated as
 * plain C: same call order (Init -> AnalyticMarching -> CombineMesh ->
 * ExportMesh, Destroy at re-initialisation or exit), same argument meaning,
 * but an explicit engine handle instead of the reference's global singleton
 * (backend/src/cuam_kernel.cu:23) and status codes instead of exit() / silent
 * prints.  Float arrays are float32 for float_type "float32" and "mixed",
 * float64 for "float64".  Every pointer argument may be host or device
 * memory; the engine detects which.  Calls on one engine must not overlap;
 * separate engines are independent.
 */
#ifndef ANALYTICMESH_GB300_H
#define ANALYTICMESH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct am_engine am_engine;

typedef enum {
    AM_OK = 0,
    AM_ERR_INVALID_ARGUMENT = 1, /* the reference: TORCH_CHECK -> RuntimeError */
    AM_ERR_NOT_INITIALIZED = 2,  /* the reference: prints and returns (cuam.cpp:107-111) */
    AM_ERR_CUDA = 3,             /* the reference: exit(code) (utilities.h:87-101) */
    AM_ERR_OUT_OF_MEMORY = 4,
    AM_ERR_TABLE_FULL = 5,       /* hash probe bound hit; the reference spins forever (hash.h:56-64) */
    AM_ERR_NO_RESULT = 6,        /* CombineMesh / ExportMesh before AnalyticMarching (cuam_kernel.cu:193-197) */
    AM_ERR_IO = 7,
    AM_ERR_CAPACITY = 8
} am_status;

/* Init -- backend/src/cuam.cpp:58-95 and backend/src/cuam_kernel.cu:128-148.
 * float_type: "float32" (plain FP32 form), "float64", or "mixed" (float32
 * inputs; tensor-core composition, FP64 vertex solves).  nodesnum: layer
 * widths including the input (3) and the output (1), at least 3 entries.
 * arc_table: (num_nodes - 2) rows x arc_cols int32, row i = connections into
 * linear layer i + 1: [count, src_0, tm_0, src_1, tm_1, ...]. */
int am_init(am_engine **engine, const char *float_type, const int32_t *nodesnum, int num_nodes,
            const int32_t *arc_table, int arc_rows, int arc_cols, int num_extra_constraints);

/* AnalyticMarching -- backend/src/cuam.cpp:97-184 and cuam_kernel.cu:104-123.
 * weights[i]: nodesnum[i+1] x nodesnum[i] row-major, biases[i]: nodesnum[i+1];
 * states: num_points x N bytes (0/1), N = sum of hidden widths;
 * points: num_points x 3; arc_tm[t]: arc_tm_shapes[2t] x arc_tm_shapes[2t+1]
 * (0 x 0 = identity); w_extra: E x 3, b_extra: E (E from am_init).
 * stream: a cudaStream_t, or NULL for the engine's own stream.  Returns when
 * the marching is complete. */
int am_analytic_marching(am_engine *engine, const void *const *weights, const void *const *biases,
                         const uint8_t *states, const void *points, int num_points, const void *const *arc_tm,
                         const int32_t *arc_tm_shapes, int num_arc_tm, const void *w_extra, const void *b_extra,
                         double iso, int flip_insideout, void *stream);

/* CombineMesh -- backend/src/cuam_kernel.cu:185-200: weld vertices, index
 * faces; output vertex = vertex * scale + center.  The weld runs on the
 * device over the polygon corners in use; the welded mesh stays in device
 * memory (moved to the host only when it passes 8 GB) until am_get_mesh
 * copies it into the caller's arrays or the next run replaces it. */
int am_combine_mesh(am_engine *engine, double scale, const double *center3);

/* ExportMesh -- backend/src/cuam_kernel.cu:205-246 (binary little-endian PLY,
 * polygons or triangle fans, float or double vertices, polymesh.h:350-423). */
int am_export_mesh(am_engine *engine, const char *file_path, int is_polymesh, int is_float32);

/* Destroy -- backend/src/cuam_kernel.cu:153-179. */
int am_destroy(am_engine *engine);

const char *am_strerror(int status);
/* Detail of the last failure on this engine (CUDA error text, which check failed). */
const char *am_last_error(const am_engine *engine);

/* ---- results: no counterpart in the reference, which only writes a PLY. */
typedef struct {
    int64_t num_regions;      /* regions visited */
    int64_t num_faces;        /* face polygons with >= 3 vertices */
    int64_t num_seeds;        /* seed regions after de-duplication */
    int64_t num_nostart;      /* seed regions without a feasible start vertex */
    int64_t num_open;         /* walks that found no closing vertex */
    int64_t num_truncated;    /* polygons that hit the vertex capacity */
    int64_t num_singular;
    int64_t mesh_num_verts;   /* after am_combine_mesh */
    int64_t mesh_num_faces;
    int64_t mesh_num_indices;
    int32_t chunks;
    int32_t max_polygon_verts;
    double am_time_ms;        /* device time of the marching loop (seeds to last chunk) */
    double compose_ms;        /* per-phase device time, when AM_OPT_PHASE_TIMING is set */
    double polygon_ms;
    double frontier_ms;
    int64_t kernel_launches;  /* launches inside the marching loop */
    /* error report: set by am_error_report, zero until it has run on this result */
    double max_abs_f;         /* max |f(v)| over the checked faces' vertices, f in FP64 */
    double max_vertex_err;    /* max |v - v64| (largest coordinate) against FP64 re-solves */
    int64_t error_faces;      /* faces checked */
    /* mixed form: faces walked again with every sign and feasibility
     * predicate in FP64, because a constraint value came within 1e-6 |w| of
     * zero at a vertex (or a decision differed between FP32 and FP64) */
    int64_t num_fp64_walks;
} am_stats;

int am_get_stats(const am_engine *engine, am_stats *out);

/* Error report of the last result (no counterpart in the reference, which
 * reports timings only, backend/main.py:368-373): sample_regions regions,
 * evenly spaced over the region store (0 or more than there are: all), are
 * composed again in FP64 from the engine's parameters (converted exactly to
 * double), and every vertex of their faces is checked: |f(v)| with f the FP64
 * face plane (the network's value at v minus the level), and the distance
 * (largest coordinate) from v to the FP64 solve of the three planes it lies
 * on.  Also stored in the am_stats fields max_abs_f, max_vertex_err and
 * error_faces.
 * Runs on the engine's stream after the marching, outside its am_time. */
typedef struct {
    int64_t faces;            /* faces checked (regions of the sample with >= 3 vertices, closed walk) */
    int64_t vertices;         /* their vertices */
    int64_t vertices_singular;/* vertices whose FP64 system is singular (left out of max_vertex_err) */
    double max_abs_f;
    double max_vertex_err;
} am_error_report_t;
int am_error_report(am_engine *engine, int64_t sample_regions, am_error_report_t *out);

/* Welded mesh after am_combine_mesh: verts mesh_num_verts x 3, face_sizes
 * mesh_num_faces, face_indices mesh_num_indices (host memory). */
int am_get_mesh(am_engine *engine, double *verts, int32_t *face_sizes, int32_t *face_indices);

/* Per-region records in region-id order (host memory, any may be NULL):
 * bits num_regions x ceil(N/32); nverts num_regions; verts num_regions x
 * vert_capacity x 3; edges num_regions x vert_capacity (plane of the edge
 * leaving each vertex); status num_regions; seeds num_regions x 3 (seed point
 * or parent edge midpoint); start num_regions (start plane, -1 for seeds). */
int am_get_regions(am_engine *engine, uint32_t *bits, int32_t *nverts, double *verts, int32_t *edges, int8_t *status,
                   double *seeds, int32_t *start);
int am_vert_capacity(void);

/* ---- batched marching of many networks (no counterpart in the reference,
 * which marches one network per Init / AnalyticMarching pair and re-Inits
 * when the architecture changes, backend/main.py:437-446).  engines[i] is an
 * engine from am_init for network i (any widths, depths, precisions); args[i]
 * holds the arguments am_analytic_marching would take for it.  Every
 * network's wave loop runs on the device on the engine's own stream, all of
 * them side by side: the waves of small networks fill the gaps the waves of
 * large ones leave.  Afterwards each engine holds its own result (am_get_stats,
 * am_combine_mesh, ...), exactly as after am_analytic_marching.  wall_ms
 * (optional) receives the device time from the first network's start to the
 * last network's end. */
typedef struct {
    const void *const *weights;
    const void *const *biases;
    const uint8_t *states;
    const void *points;
    int num_points;
    const void *const *arc_tm;
    const int32_t *arc_tm_shapes;
    int num_arc_tm;
    const void *w_extra;
    const void *b_extra;
    double iso;
    int flip_insideout;
} am_run_args;
int am_run_batch(am_engine *const *engines, const am_run_args *args, int count, double *wall_ms);

/* Constraint rows of regions [first, first + count) of the last run,
 * recomposed with the engine's composition path (no counterpart in the
 * reference, where they live only inside a batch): rows count x ALL x 4
 * (w0, w1, w2, b, sign-flipped as in backend/inc/process.h:181-192, ALL =
 * hidden units + extra constraints), eq count x 4 (face plane, b - iso). */
int am_region_rows(am_engine *engine, int64_t first, int count, double *rows, double *eq);

typedef enum {
    AM_OPT_CHUNK = 1,         /* regions per wave (default: ~2 GiB of constraint rows, whole rounds of composition tiles) */
    AM_OPT_PHASE_TIMING = 2,  /* 1: time compose / polygon / frontier separately */
    AM_OPT_WELD = 3,          /* CombineMesh vertex weld: 0 = topological (default: a vertex is named by
                                 its two edge planes and the region key without those bits, which is
                                 watertight by construction), 1 = quantised coordinates as the
                                 reference (int(v*1e6) fp32 / int(v*1e9) fp64, backend/inc/polymesh.h:192) */
    AM_OPT_GRAPH = 4,         /* 1 (default): the wave loop runs on the device as one CUDA graph with a
                                 conditional while node, no host round trip per wave; 0: host-driven loop.
                                 Phase timing always uses the host-driven loop.  Both give the same regions
                                 in the same order. */
    AM_OPT_MAX_REGIONS = 5,   /* a run that passes this many regions stops after the current wave and
                                 returns AM_ERR_CAPACITY; the regions found so far are kept and can be
                                 queried (am_get_stats, am_get_regions, am_region_rows).  0 (default):
                                 no limit */
    AM_OPT_COMPOSE_TILE = 6,  /* "mixed" composition on the tensor cores: 0 (default) automatic, 1 the
                                 operand of a tile stays in shared memory for all layers, 2 it is rebuilt
                                 per 64-deep block from the rows just written (wider tiles for layers of
                                 256 units and more), 3 as 2 with a layer's 128-row tiles multiplied in two
                                 passes, so that TMEM holds accumulators for twice as many regions (layers
                                 of 512 units).  All give the same bits. */
    AM_OPT_FACE_WARPS = 7,    /* warps per face polygon: 0 (default) automatic (one for narrow networks,
                                 up to eight for wide ones, whose rows leave room for few faces per SM),
                                 or 1, 2, 4, 8.  The warps of a face split the walk's scan over the rows. */
    AM_OPT_TABLE_SLOTS = 8,   /* region hash table: 0 (default) sized by the engine (load factor <= 1/2,
                                 grown as regions are found); n > 0: fixed at n slots rounded up to a
                                 power of two, never grown.  A run that outgrows a fixed table returns
                                 AM_ERR_TABLE_FULL when an insert reaches the probe bound, where the
                                 reference's try_insert spins forever (backend/inc/hash.h:56-64); the
                                 engine stays usable. */
    AM_OPT_INJECT_ERROR = 9,  /* test hook: device error bits (1 table full, 2 device wait limit,
                                 4 capacity, 8 non-finite parameters) written into the run's control
                                 block after the seed phase, as a kernel would leave them, so that the
                                 wave loop's error decoding can be tested without a device fault.
                                 0 (default) off; stays set until set to 0. */
    AM_OPT_PRUNE_ROWS = 10    /* 1: before walking a face, drop the constraint rows whose line provably
                                 misses the polygon (a dual-space test against a sample of the rows), so
                                 that the walk scans a few dozen rows per step instead of all; 0 (default):
                                 every row.  Both give the same faces.  Measured on GB300 the two pruning
                                 passes cost about what they save (+5 % on 3-[128]x4-1 in the mixed form,
                                 -10 to -25 % on the 1536- and 4096-row networks), hence off. */
} am_option;
int am_set_option(am_engine *engine, int option, int64_t value);

/* ---- autotuner (no counterpart in the reference): chooses AM_OPT_COMPOSE_TILE
 * (mixed form) and AM_OPT_FACE_WARPS for this engine's network architecture by
 * marching the first sample_regions regions of args once per candidate with
 * per-phase device timing (after an untimed pass), and sets them on the
 * engine.  The choice is remembered per architecture (widths, connections,
 * precision, sample size) for the life of the process; a later call for the
 * same architecture sets it without marching.  chosen (optional) receives
 * {compose tile, warps per face}.  The engine holds no marching result
 * afterwards: run am_analytic_marching. */
int am_autotune(am_engine *engine, const am_run_args *args, int64_t sample_regions, int32_t *chosen);

/* ---- self-test of the tensor-core tile used by the mixed-precision
 * composition (no counterpart in the reference): D (128 x N, fp32) =
 * A (128 x K, bf16, row-major) . B (N x K, bf16, row-major)^T on one CTA,
 * 16 <= N <= 256, N % 16 == 0, K % 64 == 0; device pointers. */
int am_selftest_umma(const void *A, const void *B, void *D, int N, int K);
/* The same tile with B staged MN-major (64-wide 128B-swizzled atoms), the
 * operand layout of the mixed composition (no counterpart in the reference);
 * the inputs and D are as for am_selftest_umma. */
int am_selftest_umma_bmn(const void *A, const void *B, void *D, int N, int K);

/* ---- region composition that allocates nothing (no counterpart in the
 * reference).  For callers that cannot let a library call cudaMalloc: code
 * whose device memory is all owned by its own pool or budget, or that runs
 * where an allocation (an implicitly synchronising call) is not allowed.
 * Plain MLP without skip connections or extra constraints, FP32.  nodesnum as
 * for am_init; weights / biases are host arrays of device pointers, weights[i]
 * (nodesnum[i+1] x nodesnum[i]) and biases[i] per linear; the other buffers
 * are on the device: states count x N bytes (0/1, N = hidden units,
 * layer-major as the reference's states), rows
 * count x N x 4 (16-byte aligned; the sign-flipped rows of
 * backend/inc/process.h:181-192), eq count x 4 (face plane, b - iso).
 * Scratch (transposed weights, packed keys) is one static 8 MiB device array
 * in the library, held by every GPU that loads it until exit; the first call
 * on each device looks its address up and should come before any stream
 * capture, and a device reset (cudaDeviceReset) makes that address stale, so
 * the entry point must not be used after one.  Calls share that array, so
 * calls that overlap on the GPU race.  A network plus states larger than the
 * array returns AM_ERR_CAPACITY; rows or eq not 16-byte aligned, or a stream
 * of another device, AM_ERR_INVALID_ARGUMENT.  A CUDA error already pending on
 * the calling thread is returned as AM_ERR_CUDA before anything is launched
 * and is not cleared. */
int am_compose_rows_noalloc(const int32_t *nodesnum, int num_nodes, const float *const *weights,
                            const float *const *biases, const uint8_t *states, int count, double iso,
                            float *rows, float *eq, void *stream);

#ifdef __cplusplus
}
#endif

#endif
