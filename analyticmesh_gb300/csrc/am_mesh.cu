// am_mesh.cu -- CombineMesh on the device: weld the vertices of all face
// polygons and index the faces.
//
// Two weld keys:
// * topological (default): a polygon vertex is the intersection of the face
//   plane with the two planes of its edges (p, q).  Every region meeting at
//   that mesh vertex differs only in the bits of p and q, so (p, q, region
//   key with bits p and q cleared) names the vertex exactly and the mesh is
//   watertight whatever the rounding of the coordinates.
// * quantised, as the reference's PolyMesh (backend/inc/polymesh.h:174-335):
//   int(v * 1e6) for fp32 data, int(v * 1e9) for fp64, compared exactly
//   rather than by a 32-bit fingerprint (polymesh.h:305).  With fp32
//   coordinates this splits vertices whose copies round to different grid
//   cells.
// Vertex / face numbering follows region order (first occurrence), so it does
// not depend on thread scheduling.  Vertices of polygons with fewer than 3
// corners are welded too, as in the reference; only polygons with 3 or more
// corners become faces.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"
#include "am_mesh.h"

namespace am {

namespace {

constexpr int kScanBlock = 1024;

__device__ __forceinline__ uint64_t qhash(const long long *q)
{
    return mix64((uint64_t)q[0] * 0x9E3779B97F4A7C15ull ^ mix64((uint64_t)q[1] + 0x632BE59BD9B4E019ull) ^
                 mix64((uint64_t)q[2] * 0xD6E8FEB86659FD93ull + 7));
}

struct VKey {
    uint64_t h;
    long long q[3]; // quantised coordinates, or (p, q, -) for the topological key
};

// planes of the two edges meeting at vertex i of region r
__device__ __forceinline__ void vertex_planes(const RegionsDev &reg, long long r, int i, int n, int &p, int &q)
{
    p = reg.edges[(size_t)r * kVMax + (i + n - 1) % n];
    q = reg.edges[(size_t)r * kVMax + i];
    if (p > q) {
        const int t = p;
        p = q;
        q = t;
    }
}

__device__ __forceinline__ uint32_t pq_mask(int w, int p, int q, int N)
{
    uint32_t m = 0u;
    if (p >= 0 && p < N && (p >> 5) == w) m |= 1u << (p & 31);
    if (q >= 0 && q < N && (q >> 5) == w) m |= 1u << (q & 31);
    return m;
}

template <typename TS>
__device__ bool make_key(const RegionsDev &reg, int mode, int N, int W, double mul, long long sid, VKey &k)
{
    const long long r = sid / kVMax;
    const int i = (int)(sid % kVMax);
    const int n = reg.nv[r];
    if (i >= n) return false;
    if (mode == 0) {
        int p, q;
        vertex_planes(reg, r, i, n, p, q);
        const uint32_t *key = reg.keys + (size_t)r * W;
        uint64_t h = reg.hash[r];
        // clear bits p and q through the additive hash, word by word
        const int wp = p >= 0 && p < N ? p >> 5 : -1, wq = q >= 0 && q < N ? q >> 5 : -1;
        if (wp >= 0) h = h - word_term(key[wp], wp) + word_term(key[wp] & ~pq_mask(wp, p, q, N), wp);
        if (wq >= 0 && wq != wp) h = h - word_term(key[wq], wq) + word_term(key[wq] & ~pq_mask(wq, p, q, N), wq);
        k.q[0] = p;
        k.q[1] = q;
        k.q[2] = 0;
        k.h = mix64(h ^ mix64(((uint64_t)(uint32_t)p << 32) | (uint32_t)q));
    } else {
        const TS *v = (const TS *)reg.verts + (size_t)sid * 3;
        k.q[0] = (long long)(int)(v[0] * (TS)mul);
        k.q[1] = (long long)(int)(v[1] * (TS)mul);
        k.q[2] = (long long)(int)(v[2] * (TS)mul);
        k.h = qhash(k.q);
    }
    return true;
}

__device__ bool same_vertex(const RegionsDev &reg, int mode, int N, int W, const VKey &a, long long sa, const VKey &b,
                            long long sb)
{
    if (a.q[0] != b.q[0] || a.q[1] != b.q[1] || a.q[2] != b.q[2]) return false;
    if (mode != 0) return true;
    const uint32_t *ka = reg.keys + (size_t)(sa / kVMax) * W;
    const uint32_t *kb = reg.keys + (size_t)(sb / kVMax) * W;
    const int p = (int)a.q[0], q = (int)a.q[1];
    for (int w = 0; w < W; ++w) {
        const uint32_t m = ~pq_mask(w, p, q, N);
        if ((ka[w] & m) != (kb[w] & m)) return false;
    }
    return true;
}

__global__ void vertex_counts_kernel(const int32_t *nv, long long R, int *cnt)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r < R) cnt[r] = min(max(nv[r], 0), kVMax);
}

// the polygon vertex slots (sid = region x kVMax + corner) in region order,
// compacted: slot j of region r is voff[r] + corner
__global__ void expand_slots_kernel(const int32_t *nv, long long R, const int *voff, long long *vsid)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int n = min(max(nv[r], 0), kVMax);
    long long *o = vsid + voff[r];
    for (int i = 0; i < n; ++i) o[i] = r * kVMax + i;
}

// the table holds compacted slot indices; the smallest index of a vertex's
// copies (the first in region order) represents it
template <typename TS>
__global__ void weld_insert_kernel(RegionsDev reg, const long long *vsid, long long V, int mode, int N, int W,
                                   unsigned long long *table, unsigned long long mask, double mul, unsigned *wslot,
                                   int *err)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= V) return;
    wslot[j] = ~0u;
    const long long sid = vsid[j];
    VKey k;
    if (!make_key<TS>(reg, mode, N, W, mul, sid, k)) return;
    unsigned long long slot = k.h & mask;
    for (int probe = 0; probe < kMaxProbes; ++probe) {
        const unsigned long long cur = atomicCAS(table + slot, kEmpty, (unsigned long long)j);
        if (cur == kEmpty) {
            wslot[j] = (unsigned)slot;
            return;
        }
        const long long osid = vsid[cur];
        VKey o;
        make_key<TS>(reg, mode, N, W, mul, osid, o);
        if (o.h == k.h && same_vertex(reg, mode, N, W, k, sid, o, osid)) {
            atomicMin(table + slot, (unsigned long long)j);
            wslot[j] = (unsigned)slot;
            return;
        }
        slot = (slot + (unsigned long long)probe + 1ull) & mask;
    }
    atomicOr(err, kErrTableFull);
}

// the representative: the table's value (the smallest index of the
// vertex's copies) at the slot where the insert found or placed the key
__global__ void weld_rep_kernel(long long V, const unsigned long long *table, const unsigned *wslot, int *rep, int *flag)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= V) return;
    const unsigned sl = wslot[j];
    const long long found = sl != ~0u ? (long long)table[sl] : -1;
    rep[j] = (int)found;
    flag[j] = (found == j) ? 1 : 0;
}

template <typename TS>
__global__ void weld_verts_kernel(RegionsDev reg, const long long *vsid, long long V, const int *rep, const int *vidx,
                                  TS scale, TS cx, TS cy, TS cz, TS *out)
{
    const long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (j >= V) return;
    if (rep[j] != j) return;
    const TS *v = (const TS *)reg.verts + (size_t)vsid[j] * 3;
    TS *o = out + (size_t)vidx[j] * 3;
    o[0] = v[0] * scale + cx;
    o[1] = v[1] * scale + cy;
    o[2] = v[2] * scale + cz;
}

__global__ void face_counts_kernel(RegionsDev reg, long long R, int *fflag, int *fsize)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int n = reg.nv[r];
    fflag[r] = n >= 3 ? 1 : 0;
    fsize[r] = n >= 3 ? n : 0;
}

__global__ void faces_kernel(RegionsDev reg, long long R, const int *voff, const int *rep, const int *vidx,
                             const int *fid, const int *foff, int flip, int *face_sizes, int *face_idx)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= R) return;
    const int n = reg.nv[r];
    if (n < 3) return;
    face_sizes[fid[r]] = n;
    int *o = face_idx + foff[r];
    const int *rp = rep + voff[r];
    for (int j = 0; j < n; ++j) {
        const int i = flip ? (n - 1 - j) : j;
        o[j] = rp[i] >= 0 ? vidx[rp[i]] : -1;
    }
}

__global__ void __launch_bounds__(kScanBlock) scan_count_kernel(const int *in, long long n, int *bsum)
{
    __shared__ int ws[32];
    const long long q = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    int v = q < n ? in[q] : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
        int s = ws[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) bsum[blockIdx.x] = s;
    }
}

__device__ int block_scan(int v, int *total)
{
    __shared__ int wsum[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int s = wsum[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        wsum[lane] = s;
    }
    __syncthreads();
    const int before = wid > 0 ? wsum[wid - 1] : 0;
    *total = wsum[31];
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kScanBlock) scan_offsets_kernel(int *bsum, long long nb, long long *total)
{
    __shared__ long long base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    for (long long b0 = 0; b0 < nb; b0 += kScanBlock) {
        const long long b = b0 + threadIdx.x;
        const int v = b < nb ? bsum[b] : 0;
        int tot;
        const int pre = block_scan(v, &tot);
        if (b < nb) bsum[b] = (int)(base + pre);
        __syncthreads();
        if (threadIdx.x == 0) base += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = base;
}

__global__ void __launch_bounds__(kScanBlock) scan_apply_kernel(const int *in, long long n, const int *bsum, int *out)
{
    const long long q = blockIdx.x * (long long)kScanBlock + threadIdx.x;
    const int v = q < n ? in[q] : 0;
    int tot;
    const int pre = block_scan(v, &tot);
    if (q < n) out[q] = bsum[blockIdx.x] + pre;
}

} // namespace

void scan_exclusive(const int *in, long long n, int *out, int *bsum, long long *d_total, cudaStream_t st)
{
    if (n <= 0) {
        cudaMemsetAsync(d_total, 0, sizeof(long long), st);
        return;
    }
    const long long nb = (n + kScanBlock - 1) / kScanBlock;
    scan_count_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, bsum);
    scan_offsets_kernel<<<1, kScanBlock, 0, st>>>(bsum, nb, d_total);
    scan_apply_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(in, n, bsum, out);
}

void launch_weld_slots(const RegionsDev &reg, long long R, const WeldBuffers &wb, cudaStream_t st)
{
    if (R <= 0) {
        cudaMemsetAsync(wb.counts, 0, sizeof(long long), st);
        return;
    }
    // vertex counts (into fflag, which the face counts overwrite later)
    vertex_counts_kernel<<<(unsigned)((R + 255) / 256), 256, 0, st>>>(reg.nv, R, wb.fflag);
    scan_exclusive(wb.fflag, R, wb.voff, wb.bsum, wb.counts + 0, st);
}

void launch_weld(int prec, int mode, int N, int W, const RegionsDev &reg, long long R, long long V,
                 const WeldBuffers &wb, double scale, const double *center, int flip, int *d_err, cudaStream_t st)
{
    const unsigned g1 = (unsigned)((V + 255) / 256);
    const unsigned g2 = (unsigned)((R + 255) / 256);
    cudaMemsetAsync(wb.table, 0xff, sizeof(unsigned long long) * (size_t)(wb.mask + 1), st);
    const bool f64 = (prec != kFloat32);
    const double mul = (prec == kFloat64) ? 1e9 : 1e6;
    if (R <= 0 || V <= 0) {
        cudaMemsetAsync(wb.counts, 0, sizeof(long long) * 3, st);
        return;
    }
    expand_slots_kernel<<<g2, 256, 0, st>>>(reg.nv, R, wb.voff, wb.vsid);
    if (f64)
        weld_insert_kernel<double><<<g1, 256, 0, st>>>(reg, wb.vsid, V, mode, N, W, wb.table, wb.mask, mul, wb.wslot,
                                                       d_err);
    else
        weld_insert_kernel<float><<<g1, 256, 0, st>>>(reg, wb.vsid, V, mode, N, W, wb.table, wb.mask, mul, wb.wslot,
                                                      d_err);
    weld_rep_kernel<<<g1, 256, 0, st>>>(V, wb.table, wb.wslot, wb.rep, wb.flag);
    scan_exclusive(wb.flag, V, wb.vidx, wb.bsum, wb.counts + 0, st);
    if (f64)
        weld_verts_kernel<double><<<g1, 256, 0, st>>>(reg, wb.vsid, V, wb.rep, wb.vidx, scale, center[0], center[1],
                                                      center[2], (double *)wb.out_verts);
    else
        weld_verts_kernel<float><<<g1, 256, 0, st>>>(reg, wb.vsid, V, wb.rep, wb.vidx, (float)scale, (float)center[0],
                                                     (float)center[1], (float)center[2], (float *)wb.out_verts);
    face_counts_kernel<<<g2, 256, 0, st>>>(reg, R, wb.fflag, wb.fsize);
    scan_exclusive(wb.fflag, R, wb.fid, wb.bsum, wb.counts + 1, st);
    scan_exclusive(wb.fsize, R, wb.foff, wb.bsum, wb.counts + 2, st);
    faces_kernel<<<g2, 256, 0, st>>>(reg, R, wb.voff, wb.rep, wb.vidx, wb.fid, wb.foff, flip, wb.face_sizes,
                                     wb.face_idx);
}

} // namespace am
