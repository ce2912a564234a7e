// am_mesh.h -- buffers of the device-side CombineMesh (weld + face indexing).
#pragma once

#include <cuda_runtime.h>

#include "am_internal.h"

namespace am {

struct WeldBuffers {
    int *voff;                  // [R] first compacted vertex slot of each region
    long long *vsid;            // [V] vertex slot (region x kVMax + corner) of each compacted slot
    unsigned long long *table;  // weld hash table (compacted slot indices)
    unsigned long long mask;
    unsigned *wslot;            // [V] table slot holding each compacted slot's key
    int *rep;                   // [V] representative compacted slot
    int *flag;                  // [V]
    int *vidx;                  // [V] output vertex index of each representative
    int *bsum;                  // scan block sums
    int *fflag, *fsize, *fid, *foff; // [R]
    void *out_verts;            // [V][3] TS
    int *face_sizes;            // [F]
    int *face_idx;              // [sum of sizes]
    long long *counts;          // [3]: V, F, total face indices
};

void scan_exclusive(const int *in, long long n, int *out, int *bsum, long long *d_total, cudaStream_t st);
// the compacted vertex slots: voff from the regions' vertex counts, their
// total V into counts[0] (read by the host before launch_weld)
void launch_weld_slots(const RegionsDev &reg, long long R, const WeldBuffers &wb, cudaStream_t st);
// mode 0: topological vertex key, 1: quantised coordinates (the reference's weld)
void launch_weld(int prec, int mode, int N, int W, const RegionsDev &reg, long long R, long long V,
                 const WeldBuffers &wb, double scale, const double *center, int flip, int *d_err, cudaStream_t st);

} // namespace am
