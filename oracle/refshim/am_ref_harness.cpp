/*
 * am_ref_harness.cpp -- C entry points around the reference's own marching
 * loop compiled for the CPU.  TEST INFRASTRUCTURE ONLY (see am_ref_shim.h).
 *
 * oracle/build_ref.py rewrites the reference's backend sources into
 * oracle/_ref/gen/ (kernel launches become OpenMP loops, see the shim) and
 * compiles this file with them into oracle/_ref/libamref.so.  The entry points
 * call the reference's Init_cuda / AnalyticMarching_cuda / CombineMesh
 * (backend/src/cuam_kernel.cu:104-200) directly; the pybind11 validation
 * layer (backend/src/cuam.cpp) is not part of the loop being measured.
 */
#include "am_ref_shim.h"

#include <chrono>
#include <omp.h>

#include "kernel.cu"
#include "states.cu"
#include "cuam_kernel.cu"

namespace {

struct HostNet {
    std::vector<int> nodes;
    std::vector<int32_t> arc;
    int arc_rows = 0, arc_cols = 0;
};
HostNet g_net;
int g_is_f64 = 0;
double g_am_seconds = 0.0;

torch::Tensor view(const void *p, int64_t d0, int64_t d1, int ndim, at::ScalarType st)
{
    torch::Tensor t;
    t.ptr = const_cast<void *>(p);
    t.sizes[0] = d0;
    t.sizes[1] = d1;
    t.ndim = ndim;
    t.st = st;
    return t;
}

} // namespace

extern "C" {

/* 1 thread runs every launch in thread-index order, which settles the
 * reference's racy choices deterministically; more threads time it. */
void amref_set_threads(int n) { omp_set_num_threads(n > 0 ? n : 1); }
int amref_get_threads(void) { return omp_get_max_threads(); }

/* Runs Init -> AnalyticMarching for one network; records every popped region.
 * Pointers are host memory in the selected float type.  Returns 0 on success. */
int amref_run(int is_f64, int n_lin, const int *nodes, const void *const *W, const void *const *b,
              const int32_t *arc_table, int arc_cols, int n_tm, const void *const *tm, const int *tm_shape, int E,
              const void *w_extra, const void *b_extra, const uint8_t *states, const void *points, int S, double iso,
              int flip)
{
    if (FloatTypeString != "") Destroy();
    g_amref_rec.clear();
    g_is_f64 = is_f64;
    at::ScalarType ft = is_f64 ? at::ScalarType::Double : at::ScalarType::Float;

    g_net.nodes.assign(nodes, nodes + n_lin + 1);
    g_net.arc_rows = n_lin - 1;
    g_net.arc_cols = arc_cols;
    g_net.arc.assign(arc_table, arc_table + (size_t)(n_lin - 1) * arc_cols);

    torch::Tensor arc = view(g_net.arc.data(), g_net.arc_rows, arc_cols, 2, at::ScalarType::Int);
    Init_cuda(is_f64 ? "float64" : "float32", g_net.nodes, arc, E);

    int N = 0;
    for (int i = 1; i < n_lin; ++i) N += nodes[i];
    std::vector<torch::Tensor> ws, bs, tms;
    for (int i = 0; i < n_lin; ++i) {
        ws.push_back(view(W[i], nodes[i + 1], nodes[i], 2, ft));
        bs.push_back(view(b[i], nodes[i + 1], 0, 1, ft));
    }
    for (int i = 0; i < n_tm; ++i) tms.push_back(view(tm[i], tm_shape[2 * i], tm_shape[2 * i + 1], 2, ft));
    torch::Tensor st = view(states, S, N, 2, at::ScalarType::Bool);
    torch::Tensor pt = view(points, S, 3, 2, ft);
    torch::Tensor we = view(w_extra, E, 3, 2, ft);
    torch::Tensor be = view(b_extra, E, 0, 1, ft);
    const auto t0 = std::chrono::steady_clock::now();
    AnalyticMarching_cuda(ws, bs, st, pt, tms, we, be, iso, flip != 0);
    g_am_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}

/* wall time of the last AnalyticMarching_cuda call (the reference's am_time window) */
double amref_last_seconds(void) { return g_am_seconds; }
/* stop after this many regions (0 = no bound) */
void amref_set_region_budget(long n) { g_amref_region_budget = n; }

int amref_num_regions(void) { return (int)g_amref_rec.nverts.size(); }
int amref_state_len(void) { return g_amref_rec.N; }
int amref_vert_max(void) { return g_amref_rec.vm; }

void amref_get_regions(uint32_t *bits, int *nverts, double *verts, int *ntab, int *tab, double *mid, int *start)
{
    const amref_records &r = g_amref_rec;
    if (bits) std::copy(r.bits.begin(), r.bits.end(), bits);
    if (nverts) std::copy(r.nverts.begin(), r.nverts.end(), nverts);
    if (verts) std::copy(r.verts.begin(), r.verts.end(), verts);
    if (ntab) std::copy(r.ntab.begin(), r.ntab.end(), ntab);
    if (tab) std::copy(r.tab.begin(), r.tab.end(), tab);
    if (mid) std::copy(r.mid.begin(), r.mid.end(), mid);
    if (start) std::copy(r.start.begin(), r.start.end(), start);
}

/* CombineMesh (cuam_kernel.cu:185-200); mesh stays in the reference's PolyMesh. */
int amref_combine(double scale, const double *center)
{
    CombineMesh(scale, std::vector<double>(center, center + 3));
    return 0;
}

int amref_mesh_num_verts(void)
{
    return g_is_f64 ? var_ptr<double>->polymesh.verts_num : var_ptr<float>->polymesh.verts_num;
}
int amref_mesh_num_faces(void)
{
    return g_is_f64 ? var_ptr<double>->polymesh.faces_num : var_ptr<float>->polymesh.faces_num;
}

/* verts: V x 3 doubles; faces: F x (1 + VERT_MAX) ints, count first */
void amref_get_mesh(double *verts, int *faces)
{
    if (g_is_f64) {
        auto &pm = var_ptr<double>->polymesh;
        for (long i = 0; i < 3L * pm.verts_num; ++i) verts[i] = pm.vertices[i];
        std::copy(pm.faces, pm.faces + (long)pm.faces_num * (1 + _VAR_VERT_MAX), faces);
    } else {
        auto &pm = var_ptr<float>->polymesh;
        for (long i = 0; i < 3L * pm.verts_num; ++i) verts[i] = pm.vertices[i];
        std::copy(pm.faces, pm.faces + (long)pm.faces_num * (1 + _VAR_VERT_MAX), faces);
    }
}

/* ExportMesh (cuam_kernel.cu:205-246) */
int amref_export(const char *path, int is_polymesh, int is_float32)
{
    ExportMesh(std::string(path), is_polymesh != 0, is_float32 != 0);
    return 0;
}

void amref_destroy(void)
{
    if (FloatTypeString != "") Destroy();
    g_amref_rec.clear();
}

} /* extern "C" */
