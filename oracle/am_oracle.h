/*
 * am_oracle.h -- CPU restatement of the reference Analytic Marching loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * CUDA engine in analyticmesh_gb300/.  Only tests/, __graft_entry__.smoke()
 * and bench.py's cpu_baseline / --impl reference legs may load it.  The
 * product path never links, imports or executes anything under oracle/.
 *
 * Parity pin: the restatement is checked against the reference's own
 * sources compiled for the CPU (oracle/build_ref.py -> oracle/_ref/) on
 * identical inputs, see tests/test_oracle_pin.py.
 *
 * What it restates (paths relative to the reference project root):
 *   backend/src/cuam_kernel.cu:30-100   main_ batch loop (LIFO batches of 1024)
 *   backend/inc/process.h:18-193        fill_constraints (region affine composition)
 *   backend/inc/process.h:198-264       offset_b_equ, fill_distance, sortDistance
 *   backend/inc/kernel.h:609-856        calcStartIdx (pair enumeration, 3x3 solve, feasibility)
 *   backend/inc/kernel.h:861-1320       calcPivoting (polygon walk)
 *   backend/inc/kernel.h:1325-1385      correctNormalDirection
 *   backend/inc/kernel.h:1390-1506      inferNewStates
 *   backend/inc/hash.h:33-67, backend/src/states.cu:11-26   FNV hash set
 *   backend/inc/states.h:147-282        seed de-duplication, LIFO stack
 *   backend/inc/polymesh.h:120-346      raw polygon append, vertex weld, face indexing
 *
 * The reference runs one GPU thread per work item and resolves some choices
 * by races (start edge: last writer wins, kernel.cu:80-101; pivot candidate:
 * first thread to take the per-region mutex wins, kernel.h:1179).  This
 * restatement processes the work items in thread-index order, so it picks
 * the candidate with the lowest enumeration index; with full batches of
 * 1024 regions the reference does the same, because each region then gets
 * exactly one candidate per round.
 */
#ifndef AM_ORACLE_H
#define AM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AMO_VERT_MAX 20      /* backend/inc/macro.h:41 _VAR_VERT_MAX */
#define AMO_BATCH_MAX 1024   /* backend/inc/macro.h:39 _VAR_BATCH_SIZE_MAX */
#define AMO_SOLVE_MAX 1024   /* backend/inc/macro.h:40 _VAR_SOLVE_SIZE_MAX */

typedef struct {
    int n_lin;                  /* number of linear layers = len(nodes) - 1 */
    const int *nodes;           /* len n_lin + 1; nodes[0] == 3, nodes[n_lin] == 1 */
    const void *const *W;       /* W[i]: nodes[i+1] x nodes[i], row-major, REAL */
    const void *const *b;       /* b[i]: nodes[i+1] */
    const int *arc_table;       /* (n_lin - 1) x arc_cols, row-major int32 */
    int arc_cols;
    int n_tm;                   /* transform matrices */
    const void *const *tm;      /* tm[i]: tm_shape[2i] x tm_shape[2i+1]; (0,0) = identity */
    const int *tm_shape;
    int E;                      /* extra constraints */
    const void *w_extra;        /* E x 3 */
    const void *b_extra;        /* E */
    int output_skips;           /* 0: connections into the output layer are ignored,
                                   as fill_constraints does (process.h:41-178) */
} amo_net;

typedef struct amo_result amo_result;

/* Run the full marching loop.  states: S x N bytes (0/1), points: S x 3 REAL.
 * Returns 0 on success. */
int amo_run_f32(const amo_net *net, const uint8_t *states, const float *points, int S,
                double iso, int flip_insideout, amo_result **out);
int amo_run_f64(const amo_net *net, const uint8_t *states, const double *points, int S,
                double iso, int flip_insideout, amo_result **out);

/* Region records, in processing order (one per popped state). */
int amo_num_regions(const amo_result *r);
int amo_state_len(const amo_result *r);   /* N (hidden units) */
int amo_num_seeds_kept(const amo_result *r);
/* bits: R x ceil(N/32) uint32; nverts: R; verts: R x VERT_MAX x 3 (double);
 * ntab: R; tab: R x (VERT_MAX + 1); mid: R x 3; start: R (start_idx after the
 * start search). Any pointer may be NULL. */
void amo_get_regions(const amo_result *r, uint32_t *bits, int *nverts, double *verts,
                     int *ntab, int *tab, double *mid, int *start);

/* CombineMesh (polymesh.h:339-346): weld + index.  Returns 0 on success. */
int amo_combine(amo_result *r, double scale, const double *center);
int amo_mesh_num_verts(const amo_result *r);
int amo_mesh_num_faces(const amo_result *r);
/* verts: V x 3; faces: F x (1 + VERT_MAX) with count first */
void amo_get_mesh(const amo_result *r, double *verts, int *faces);

void amo_free(amo_result *r);

/* Timed samples: stop the marching loop at the end of the first batch after
 * which `regions` regions have been recorded (0 = run to completion). */
void amo_set_region_budget(long regions);

/* FNV helpers (states.cu:11-26), exported for tests. */
uint32_t amo_fnv1a(const uint8_t *data, int n);
uint32_t amo_fnv1(const uint8_t *data, int n);
/* get_i_j pair enumeration (kernel.h:607-622), exported for tests. */
void amo_get_i_j(int x, int ij_max, int *i, int *j);

#ifdef __cplusplus
}
#endif

#endif
