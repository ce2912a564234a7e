// am_internal.h -- shared types of the GB300 Analytic Marching engine
// (host driver <-> kernels).  Not part of the C ABI.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace am {

constexpr int kMaxLayers = 24;   // linear layers
constexpr int kMaxSkips = 4;     // additive connections into one layer
constexpr int kVMax = 32;        // polygon capacity (vertices / edges per face)
constexpr int kWalkSteps = 96;   // bound on walk iterations (vertices + merges)
constexpr int kTopK = 64;        // seed start search: pairs x <= 812 use the 57 nearest planes
constexpr int kMaxProbes = 4096; // hash probe bound
constexpr uint64_t kEmpty = ~0ull;
constexpr int kMaxWaves = 1 << 20; // bound on the waves of one graph launch

enum Precision : int { kFloat32 = 0, kFloat64 = 1, kMixed = 2 };

// Region status codes (poly_status)
enum : int8_t { kOk = 0, kNoStart = 1, kOpen = 2, kTruncated = 3, kSingular = 4 };

// Device error bits.  kErrWait: a bounded wait inside a kernel (a
// tensor-core pipeline barrier) ran out; the kernel stopped issuing work and
// returned, and its results are not valid.  kErrNonFinite: a weight, bias,
// transform or extra constraint is NaN or infinite.
enum : int { kErrTableFull = 1, kErrWait = 2, kErrCapacity = 4, kErrNonFinite = 8 };

struct SkipDev {
    int from;        // 0 = network input, h >= 1 = hidden layer h
    int kind;        // 0 identity, 1 transform
    const void *tmt; // transform, transposed and padded: [dec][Mp]
    int Mp;
};

// A network resident on the device in the layouts the kernels read.
struct NetDev {
    int n_lin;                    // linear layers
    int N, E, ALL, ALLP, W;       // hidden units, extra rows, N+E, padded, key words
    int nodes[kMaxLayers + 1];
    int hoff[kMaxLayers + 1];     // first constraint row of hidden layer h (h >= 1)
    const void *Wt[kMaxLayers];   // linear i transposed and padded: [nodes[i]][Mp[i]]
    int Mp[kMaxLayers];
    const void *bias[kMaxLayers]; // [nodes[i+1]]
    const void *W0;               // linear 0 as given: [nodes[1]][3]
    int nskip[kMaxLayers];        // connections into linear i
    SkipDev skip[kMaxLayers][kMaxSkips];
    const void *w_extra;          // [E][3]
    const void *b_extra;          // [E]
};

// Region store: append-only, indexed by region id (rid).
struct RegionsDev {
    uint32_t *keys;     // [cap][W] packed activation bits
    uint64_t *hash;     // [cap]
    void *mid;          // [cap][4] TS: seed point / edge midpoint
    int32_t *start;     // [cap] start plane (-1 = seed)
    int32_t *nv;        // [cap] polygon vertex count
    int8_t *status;     // [cap]
    void *verts;        // [cap][kVMax][3] TS
    int32_t *edges;     // [cap][kVMax] plane of the edge leaving vertex i
    long long cap;
};

struct HashDev {
    unsigned long long *slots;
    unsigned long long mask;
};

// Wave control block in device memory.  The host-driven loop reads tail and
// err after every wave; the graph-driven loop keeps head and count here too,
// so the kernels of a captured wave read their range from the device and a
// one-thread step kernel advances the queue and decides whether to go on.
struct WaveCtl {
    long long tail;     // regions in the store (appends advance it)
    int err;            // device error bits
    int pad0;
    long long head;     // first region of the current wave (graph-driven loop)
    int count;          // regions in the current wave
    int waves;          // waves completed
    long long limit;    // go on only while tail + count * kVMax <= limit
    int chunk_cap;      // largest wave
    unsigned int work;  // next region of the wave for the polygon warps
    int max_waves;      // waves one graph launch may run
    int grow_at;        // stop while more regions than this wait (a batch member's wave buffers grow with its queue)
    long long stop_tail; // stop after the wave that takes tail past this (a region limit)
};

// the control block's device / pinned allocation: WaveCtl, then the run's
// statistics counters (faces, largest polygon, then one count per status
// kNoStart .. kSingular, reduced at the end of a run), then the count of
// faces walked again with FP64 predicates (accumulated during the run)
constexpr int kStatsCount = 6;
constexpr int kFp64Slot = kStatsCount;
constexpr size_t kStatsOff = (sizeof(WaveCtl) + 15) / 16 * 16;
constexpr size_t kCtlBytes = kStatsOff + (kStatsCount + 1) * sizeof(unsigned long long);

struct ChunkDev {
    long long head;     // first rid of the chunk
    int count;          // regions in the chunk
    void *cons;         // [count][ALLP][4] TC constraint rows
    void *eq;           // [count][4] TC face plane (b already offset by iso)
    int32_t *rec;       // [count * kVMax] hash slot claimed by each child, -1 none
    WaveCtl *ctl = nullptr; // set: head and count come from the device (graph-driven loop)
};

#ifdef __CUDACC__
// the wave's range, from the launch or from the device
__device__ __forceinline__ void chunk_range(const ChunkDev &ch, long long &head, int &count)
{
    if (ch.ctl) {
        head = *(volatile const long long *)&ch.ctl->head;
        count = *(volatile const int *)&ch.ctl->count;
    } else {
        head = ch.head;
        count = ch.count;
    }
}
#endif

struct Tolerances {
    double eps;         // feasibility (geometric distance), reference FP_EPS
    double same_eps;    // vertex merge (L1), reference FP_SAME_EPS
    double par_eps;     // a plane counts as crossing an edge line when w.d > par_eps |w| |d|
};

// launchers (stream-ordered, no synchronisation)
void launch_compose(int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, double iso,
                    cudaStream_t st);
// prune: 1 = the walk scans only the rows that can bound the face (see
// prune_rows), 0 = every row (the same faces)
// nfp64: counts the faces the mixed form walks again with FP64 predicates
void launch_polygon(int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, const HashDev &hs,
                    const Tolerances &tol, int face_warps, int prune, unsigned long long *nfp64, int *d_err,
                    cudaStream_t st);
int polygon_face_warps(int prec, int ALLP);
void launch_seed_pack(const uint8_t *states, int S, int N, int W, uint32_t *keys, uint64_t *hash, cudaStream_t st);
void launch_seed_insert(const uint32_t *keys, const uint64_t *hash, int S, int W, const HashDev &hs, int32_t *rec,
                        int *d_err, cudaStream_t st);
// flags + scan + append.  mode 0: children of a chunk, mode 1: seeds.
void launch_append(int mode, int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch,
                   const HashDev &hs, const uint32_t *seed_keys, const uint64_t *seed_hash, const void *seed_points,
                   int n_items, long long *d_tail, int *d_blocksum, int nblocks_cap, int *d_err, cudaStream_t st);
void launch_rehash(const RegionsDev &reg, long long n, const HashDev &hs, int *d_err, cudaStream_t st);
// graph-driven loop: advance ctl to the next wave and set the loop condition
void launch_region_stats(const int32_t *nv, const int8_t *status, long long n, unsigned long long *out,
                         cudaStream_t st);
void launch_wave_step(WaveCtl *ctl, cudaGraphConditionalHandle cond, cudaStream_t st);
int device_sms();
// the network's parameter buffers, checked for NaN / infinity in one launch
struct FiniteList {
    const void *p[64];
    long long n[64];
    int count;
};
void launch_check_finite(int prec, const FiniteList &list, int *d_err, cudaStream_t st);
void launch_prepare_weights(int prec, const void *src, int M, int K, int Mp, void *dst, cudaStream_t st);

// error report (am_verify.cu): out[0] max |f(v)| bits, out[1] max vertex
// error bits, out[2] vertices, out[3] vertices left out (singular), out[4] faces
void launch_gather_keys(const uint32_t *keys, int W, const long long *ids, int count, uint32_t *out, cudaStream_t st);
void launch_to_double(const void *src, long long n, void *dst, cudaStream_t st);
void launch_verify(int ts_bytes, const RegionsDev &reg, const long long *ids, int count, const double *rows,
                   const double *eq, int ALLP, int ALL, unsigned long long *out, cudaStream_t st);

// mesh weld (CombineMesh)
struct MeshDev {
    unsigned long long *vslots; // weld table: packed (vertex slot id) per hash slot
    unsigned long long vmask;
    int64_t *vkey;              // [nslots_total][2] quantised key per vertex slot (x,y | z)
};

} // namespace am
