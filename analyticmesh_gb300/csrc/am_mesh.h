// am_mesh.h -- buffers of the device-side CombineMesh (weld + face indexing).
#pragma once

#include <cuda_runtime.h>

#include "am_internal.h"

namespace am {

struct WeldBuffers {
    unsigned long long *table;  // weld hash table
    unsigned long long mask;
    long long *rep;             // [R * kVMax] representative vertex slot
    int *flag;                  // [R * kVMax]
    int *vidx;                  // [R * kVMax] output vertex index of each representative
    int *bsum;                  // scan block sums
    int *fflag, *fsize, *fid, *foff; // [R]
    void *out_verts;            // [V][3] TS
    int *face_sizes;            // [F]
    int *face_idx;              // [sum of sizes]
    long long *counts;          // [3]: V, F, total face indices
};

void scan_exclusive(const int *in, long long n, int *out, int *bsum, long long *d_total, cudaStream_t st);
// mode 0: topological vertex key, 1: quantised coordinates (the reference's weld)
void launch_weld(int prec, int mode, int N, int W, const RegionsDev &reg, long long R, const WeldBuffers &wb,
                 double scale, const double *center, int flip, int *d_err, cudaStream_t st);

} // namespace am
