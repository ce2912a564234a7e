/*
 * am_oracle.c -- CPU restatement of the reference Analytic Marching loop.
 * TEST INFRASTRUCTURE ONLY (see am_oracle.h).  Build with -ffp-contract=off
 * so the x86 and Arm builds round identically.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "am_oracle.h"

struct amo_result {
    int N, words, is_f64, seeds_kept;
    long num, cap;
    uint32_t *bits;
    int *nverts;
    double *verts;
    int *ntab;
    int *tab;
    double *mid;
    int *start;
    int mesh_nv, mesh_nf;
    double *mverts;
    int *mfaces;
};

/* Region budget for timed samples: 0 = none; otherwise the loop stops at the
 * end of the first batch after which this many regions have been recorded
 * (the same point as the hook of the reference's CPU build). */
static long g_region_budget = 0;

void amo_set_region_budget(long regions) { g_region_budget = regions > 0 ? regions : 0; }

/* FNV-1a (hash1) and FNV-1 (hash2), 32-bit, backend/src/states.cu:11-26 */
uint32_t amo_fnv1a(const uint8_t *data, int n)
{
    uint32_t h = 0x811C9DC5u;
    while (n--) h = (h ^ (*data++)) * 0x01000193u;
    return h;
}

uint32_t amo_fnv1(const uint8_t *data, int n)
{
    uint32_t h = 0x811C9DC5u;
    while (n--) h = (h * 0x01000193u) ^ (*data++);
    return h;
}

/* get_i_j, backend/inc/kernel.h:607-622: x >= 0 -> pair (i, j), i > j,
 * enumerated along anti-diagonals of i + j, clamped to ij_max - 1. */
void amo_get_i_j(int x, int ij_max, int *pi, int *pj)
{
    int k = x / 2;
    int a = (int)ceilf(sqrtf(2 * k + 2.25f) - 1.5f);
    int r = x - a * (a + 1);
    int A = 2 * a + r / (a + 1);
    int B = r % (a + 1);
    int i = (A + 1) / 2 + B + 1;
    int j = A + 1 - i;
    *pi = (i < ij_max ? i : (ij_max - 1));
    *pj = (j < ij_max ? j : (ij_max - 1));
}

static inline float amo_sqrt_f32(float x) { return sqrtf(x); }
static inline double amo_sqrt_f64(double x) { return sqrt(x); }
static inline float amo_fabs_f32(float x) { return fabsf(x); }
static inline double amo_fabs_f64(double x) { return fabs(x); }

/* float instantiation: macro.h:17,20,23 */
#define REAL float
#define SFX _f32
#define R_EPS (1e-12f)
#define R_SAME_EPS (3e-7f)
#define R_PH_MUL 1000000
#include "am_oracle_impl.h"
#undef REAL
#undef SFX
#undef R_EPS
#undef R_SAME_EPS
#undef R_PH_MUL

/* double instantiation: macro.h:18,21,24 */
#define REAL double
#define SFX _f64
#define R_EPS (1e-20)
#define R_SAME_EPS (3e-14)
#define R_PH_MUL 1000000000
#include "am_oracle_impl.h"
#undef REAL
#undef SFX
#undef R_EPS
#undef R_SAME_EPS
#undef R_PH_MUL

int amo_run_f32(const amo_net *net, const uint8_t *states, const float *points, int S, double iso, int flip,
                amo_result **out)
{
    return run_f32(net, states, points, S, iso, flip, out);
}

int amo_run_f64(const amo_net *net, const uint8_t *states, const double *points, int S, double iso, int flip,
                amo_result **out)
{
    return run_f64(net, states, points, S, iso, flip, out);
}

int amo_num_regions(const amo_result *r) { return (int)r->num; }
int amo_state_len(const amo_result *r) { return r->N; }
int amo_num_seeds_kept(const amo_result *r) { return r->seeds_kept; }

void amo_get_regions(const amo_result *r, uint32_t *bits, int *nverts, double *verts, int *ntab, int *tab, double *mid,
                     int *start)
{
    const size_t n = (size_t)r->num;
    if (bits) memcpy(bits, r->bits, sizeof(uint32_t) * n * (size_t)r->words);
    if (nverts) memcpy(nverts, r->nverts, sizeof(int) * n);
    if (verts) memcpy(verts, r->verts, sizeof(double) * n * AMO_VERT_MAX * 3);
    if (ntab) memcpy(ntab, r->ntab, sizeof(int) * n);
    if (tab) memcpy(tab, r->tab, sizeof(int) * n * (AMO_VERT_MAX + 1));
    if (mid) memcpy(mid, r->mid, sizeof(double) * n * 3);
    if (start) memcpy(start, r->start, sizeof(int) * n);
}

int amo_combine(amo_result *r, double scale, const double *center)
{
    return r->is_f64 ? combine_f64(r, scale, center) : combine_f32(r, scale, center);
}

int amo_mesh_num_verts(const amo_result *r) { return r->mesh_nv; }
int amo_mesh_num_faces(const amo_result *r) { return r->mesh_nf; }

void amo_get_mesh(const amo_result *r, double *verts, int *faces)
{
    if (verts) memcpy(verts, r->mverts, sizeof(double) * 3 * (size_t)r->mesh_nv);
    if (faces) memcpy(faces, r->mfaces, sizeof(int) * (size_t)r->mesh_nf * (1 + AMO_VERT_MAX));
}

void amo_free(amo_result *r)
{
    if (!r) return;
    free(r->bits); free(r->nverts); free(r->verts); free(r->ntab); free(r->tab);
    free(r->mid); free(r->start); free(r->mverts); free(r->mfaces);
    free(r);
}
