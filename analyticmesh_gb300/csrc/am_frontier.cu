// am_frontier.cu -- region hash set and the append-only region store.
//
// The reference keeps visited regions as 32-bit FNV-1 fingerprints in an
// open-addressing table and accepts a region as new when its fingerprint is
// absent (backend/inc/hash.h:33-67) -- two different regions with the same
// fingerprint silently lose one.  This store keeps every region's full
// packed key; a table slot holds (fingerprint, id) and a fingerprint match
// is confirmed by comparing the keys.
//
// New regions are appended in candidate order: winners of the insert are
// flagged and counted per block; each block then writes its winners at the
// tail plus the counts of the blocks before it, so the region ids of a run do
// not depend on thread scheduling.
#include <algorithm>
#include <cuda/atomic>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"

namespace am {

namespace {

constexpr int kScanBlock = 1024;

__device__ __forceinline__ unsigned long long load_slot(const unsigned long long *p)
{
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*const_cast<unsigned long long *>(p));
    return a.load(cuda::memory_order_relaxed);
}

// Exclusive scan over the block; returns this thread's prefix, writes the total.
__device__ int block_exclusive_scan(int v, int *total)
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
        const int nw = blockDim.x >> 5;
        int s = lane < nw ? wsum[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) wsum[lane] = s;
    }
    __syncthreads();
    const int before = wid > 0 ? wsum[wid - 1] : 0;
    *total = wsum[(blockDim.x >> 5) - 1];
    __syncthreads();
    return before + x - v;
}

__global__ void seed_pack_kernel(const uint8_t *states, int S, int N, int W, uint32_t *keys, uint64_t *hash)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint8_t *row = states + (size_t)s * N;
    uint64_t h = 0;
    for (int w = 0; w < W; ++w) {
        uint32_t word = 0;
        const int lim = min(32, N - 32 * w);
        for (int b = 0; b < lim; ++b)
            if (row[32 * w + b]) word |= 1u << b;
        keys[(size_t)s * W + w] = word;
        h += word_term(word, w);
    }
    hash[s] = h;
}

__global__ void seed_insert_kernel(const uint32_t *keys, const uint64_t *hash, int S, int W, HashDev hs, int32_t *rec,
                                   int *err)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= S) return;
    const uint64_t h = hash[s];
    const uint32_t fp = fp_of(h);
    const unsigned long long mine = slot_value(fp, 1, (uint32_t)s);
    const uint32_t *key = keys + (size_t)s * W;
    unsigned long long slot = h & hs.mask;
    int r = -1, probe = 0;
    for (; probe < kMaxProbes; ++probe) {
        unsigned long long cur = load_slot(hs.slots + slot);
        if (cur == kEmpty) {
            const unsigned long long old = atomicCAS(hs.slots + slot, kEmpty, mine);
            if (old == kEmpty) {
                r = (int)slot;
                break;
            }
            cur = old;
        }
        if ((uint32_t)(cur >> 32) == fp) {
            const uint32_t *other = keys + (size_t)((uint32_t)cur & 0x7fffffffu) * W;
            bool eq = true;
            for (int w = 0; w < W && eq; ++w) eq = (other[w] == key[w]);
            if (eq) {
                atomicMin(hs.slots + slot, mine);
                r = (int)slot;
                break;
            }
        }
        slot = (slot + (unsigned long long)probe + 1ull) & hs.mask;
    }
    if (probe == kMaxProbes) atomicOr(err, kErrTableFull);
    rec[s] = r;
}

struct AppendArgs {
    int mode;              // 0 children of a chunk, 1 seeds
    NetDev net;
    RegionsDev reg;
    ChunkDev ch;
    HashDev hs;
    const uint32_t *seed_keys;
    const uint64_t *seed_hash;
    const void *seed_points; // [S][3] TS
    int n_items;
    long long *tail;
    int *blockoff;         // winners per block
    long long *base;       // the tail before this append (written by the count pass)
    int *err;
};

// items of this append: head of the chunk and the number of candidates, from
// the launch or (graph-driven loop) from the wave control block
__device__ __forceinline__ void append_range(const AppendArgs &a, long long &head, int &n)
{
    if (a.ch.ctl) {
        head = *(volatile const long long *)&a.ch.ctl->head;
        n = *(volatile const int *)&a.ch.ctl->count * kVMax;
    } else {
        head = a.ch.head;
        n = a.n_items;
    }
}

// block b scans items [b * span, (b + 1) * span) in tiles of kScanBlock
__device__ __forceinline__ int block_span(int n)
{
    const int tiles = (n + kScanBlock - 1) / kScanBlock;
    return (tiles + (int)gridDim.x - 1) / (int)gridDim.x * kScanBlock;
}

__device__ __forceinline__ int is_winner(const AppendArgs &a, int q, long long head, int n)
{
    if (q >= n) return 0;
    const int rec = a.ch.rec[q];
    if (rec < 0) return 0;
    uint32_t myid;
    if (a.mode == 1) {
        myid = (uint32_t)q;
    } else {
        const long long rl = q / kVMax;
        const int i = q % kVMax;
        const int k = a.reg.edges[(size_t)(head + rl) * kVMax + i];
        myid = (uint32_t)(rl * a.net.ALL + k);
    }
    const unsigned long long cur = load_slot(a.hs.slots + rec);
    return ((uint32_t)cur == ((1u << 31) | (myid & 0x7fffffffu))) ? 1 : 0;
}

__global__ void __launch_bounds__(kScanBlock) append_count_kernel(AppendArgs a)
{
    long long head;
    int n;
    append_range(a, head, n);
    const int span = block_span(n);
    const int q1 = min(n, (int)blockIdx.x * span + span);
    int sum = 0;
    for (int q0 = (int)blockIdx.x * span; q0 < q1; q0 += kScanBlock) {
        int total;
        block_exclusive_scan(is_winner(a, q0 + (int)threadIdx.x, head, n), &total);
        sum += total;
    }
    if (threadIdx.x == 0) a.blockoff[blockIdx.x] = sum;
    if (blockIdx.x == 0 && threadIdx.x == 0) *a.base = *a.tail;
}

template <typename TS>
__device__ void append_one(const AppendArgs &a, int q, long long rid, long long head)
{
    if (rid >= a.reg.cap) {
        atomicOr(a.err, kErrCapacity);
        return;
    }
    const int W = a.net.W;
    uint32_t *key = a.reg.keys + (size_t)rid * W;
    TS *mid = (TS *)a.reg.mid + (size_t)rid * 4;
    uint64_t h;
    if (a.mode == 1) {
        const uint32_t *sk = a.seed_keys + (size_t)q * W;
        for (int w = 0; w < W; ++w) key[w] = sk[w];
        h = a.seed_hash[q];
        const TS *pt = (const TS *)a.seed_points + (size_t)q * 3;
        mid[0] = pt[0];
        mid[1] = pt[1];
        mid[2] = pt[2];
        mid[3] = TS(0);
        a.reg.start[rid] = -1;
    } else {
        const long long parent = head + q / kVMax;
        const int i = q % kVMax;
        const int k = a.reg.edges[(size_t)parent * kVMax + i];
        const uint32_t *pk = a.reg.keys + (size_t)parent * W;
        for (int w = 0; w < W; ++w) key[w] = pk[w];
        key[k >> 5] ^= 1u << (k & 31);
        h = flip_hash(a.reg.hash[parent], pk[k >> 5], k);
        const int n = a.reg.nv[parent];
        const TS *v0 = (const TS *)a.reg.verts + ((size_t)parent * kVMax + i) * 3;
        const TS *v1 = (const TS *)a.reg.verts + ((size_t)parent * kVMax + (i + 1) % n) * 3;
        mid[0] = (v0[0] + v1[0]) / TS(2);
        mid[1] = (v0[1] + v1[1]) / TS(2);
        mid[2] = (v0[2] + v1[2]) / TS(2);
        mid[3] = TS(0);
        a.reg.start[rid] = k;
    }
    a.reg.hash[rid] = h;
    a.reg.nv[rid] = 0;
    a.reg.status[rid] = 0;
    a.hs.slots[a.ch.rec[q]] = slot_value(fp_of(h), 0, (uint32_t)rid);
}

// Appends this block's winners after the winners of every block before it
// (the block sums them itself: at most a few thousand counts); the last
// block moves the tail.
template <typename TS>
__global__ void __launch_bounds__(kScanBlock) append_write_kernel(AppendArgs a)
{
    long long head;
    int n;
    append_range(a, head, n);
    int part = 0;
    for (int b = threadIdx.x; b < (int)blockIdx.x; b += kScanBlock) part += a.blockoff[b];
    int before;
    block_exclusive_scan(part, &before); // (its total: the winners of every earlier block)
    long long base = *a.base + before;
    const int span = block_span(n);
    const int q1 = min(n, (int)blockIdx.x * span + span);
    for (int q0 = (int)blockIdx.x * span; q0 < q1; q0 += kScanBlock) {
        const int q = q0 + (int)threadIdx.x;
        int total;
        const int f = is_winner(a, q, head, n);
        const int pre = block_exclusive_scan(f, &total);
        if (f) append_one<TS>(a, q, base + pre, head);
        base += total;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) *a.tail = base;
}

// graph-driven loop: retire the wave, take the next one from the queue and
// go on while it is non-empty, no error bit is set, its children fit and the
// queue has not outgrown the wave buffers of a batch member
__global__ void wave_step_kernel(WaveCtl *ctl, cudaGraphConditionalHandle cond)
{
    WaveCtl &c = *ctl;
    if (c.count > 0) c.waves++;
    c.head += c.count;
    const long long rem = c.tail - c.head;
    c.count = (int)(rem < (long long)c.chunk_cap ? (rem > 0 ? rem : 0) : (long long)c.chunk_cap);
    c.work = 0u;
    const bool go = c.count > 0 && c.err == 0 &&
                    c.tail + (long long)c.count * kVMax <= c.limit && c.waves < c.max_waves &&
                    c.tail <= c.stop_tail && rem <= (long long)c.grow_at;
    cudaGraphSetConditional(cond, go ? 1u : 0u);
}

// run statistics: faces (>= 3 vertices), the largest polygon, and one count
// per failure status
__global__ void region_stats_kernel(const int32_t *nv, const int8_t *status, long long n, unsigned long long *out)
{
    __shared__ unsigned int s[kStatsCount];
    if (threadIdx.x < kStatsCount) s[threadIdx.x] = 0u;
    __syncthreads();
    unsigned int faces = 0, vmax = 0, bad[4] = {0u, 0u, 0u, 0u};
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += (long long)gridDim.x * blockDim.x) {
        const int v = nv[r];
        faces += v >= 3 ? 1u : 0u;
        vmax = max(vmax, (unsigned int)max(v, 0));
        const int st = status[r];
        if (st >= kNoStart && st <= kSingular) bad[st - kNoStart]++;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        faces += __shfl_xor_sync(0xffffffffu, faces, o);
        vmax = max(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
#pragma unroll
        for (int b = 0; b < 4; ++b) bad[b] += __shfl_xor_sync(0xffffffffu, bad[b], o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&s[0], faces);
        atomicMax(&s[1], vmax);
        for (int b = 0; b < 4; ++b) atomicAdd(&s[2 + b], bad[b]);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        atomicAdd(out, (unsigned long long)s[0]);
        atomicMax(out + 1, (unsigned long long)s[1]);
        for (int b = 0; b < 4; ++b) atomicAdd(out + 2 + b, (unsigned long long)s[2 + b]);
    }
}

__global__ void rehash_kernel(RegionsDev reg, long long n, HashDev hs, int *err)
{
    const long long rid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (rid >= n) return;
    const uint64_t h = reg.hash[rid];
    const unsigned long long v = slot_value(fp_of(h), 0, (uint32_t)rid);
    unsigned long long slot = h & hs.mask;
    for (int probe = 0; probe < kMaxProbes; ++probe) {
        if (atomicCAS(hs.slots + slot, kEmpty, v) == kEmpty) return;
        slot = (slot + (unsigned long long)probe + 1ull) & hs.mask;
    }
    atomicOr(err, kErrTableFull);
}

} // namespace

void launch_seed_pack(const uint8_t *states, int S, int N, int W, uint32_t *keys, uint64_t *hash, cudaStream_t st)
{
    if (S <= 0) return;
    seed_pack_kernel<<<(S + 127) / 128, 128, 0, st>>>(states, S, N, W, keys, hash);
}

void launch_seed_insert(const uint32_t *keys, const uint64_t *hash, int S, int W, const HashDev &hs, int32_t *rec,
                        int *d_err, cudaStream_t st)
{
    if (S <= 0) return;
    seed_insert_kernel<<<(S + 127) / 128, 128, 0, st>>>(keys, hash, S, W, hs, rec, d_err);
}

void launch_append(int mode, int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, const HashDev &hs,
                   const uint32_t *seed_keys, const uint64_t *seed_hash, const void *seed_points, int n_items,
                   long long *d_tail, int *d_blocksum, int nblocks_cap, int *d_err, cudaStream_t st)
{
    if (n_items <= 0) return;
    AppendArgs a;
    a.mode = mode;
    a.net = net;
    a.reg = reg;
    a.ch = ch;
    a.hs = hs;
    a.seed_keys = seed_keys;
    a.seed_hash = seed_hash;
    a.seed_points = seed_points;
    a.n_items = n_items; // graph-driven loop: the largest wave's candidates
    a.tail = d_tail;
    a.blockoff = d_blocksum;
    a.err = d_err;
    int nb = (n_items + kScanBlock - 1) / kScanBlock;
    if (ch.ctl) nb = std::min(nb, 2 * device_sms()); // several tiles per block
    // d_blocksum: nb block counts, then (8-byte aligned) the tail snapshot
    const int base_slot = (nblocks_cap - 2) & ~1;
    if (nb > base_slot) { // the host sizes d_blocksum for the largest chunk
        int e = kErrCapacity;
        cudaMemcpyAsync(d_err, &e, sizeof(int), cudaMemcpyHostToDevice, st);
        return;
    }
    a.base = reinterpret_cast<long long *>(d_blocksum + base_slot);
    append_count_kernel<<<nb, kScanBlock, 0, st>>>(a);
    if (prec == kFloat32)
        append_write_kernel<float><<<nb, kScanBlock, 0, st>>>(a);
    else
        append_write_kernel<double><<<nb, kScanBlock, 0, st>>>(a);
}

void launch_wave_step(WaveCtl *ctl, cudaGraphConditionalHandle cond, cudaStream_t st)
{
    wave_step_kernel<<<1, 1, 0, st>>>(ctl, cond);
}

void launch_region_stats(const int32_t *nv, const int8_t *status, long long n, unsigned long long *out,
                         cudaStream_t st)
{
    if (n <= 0) return;
    const int grid = (int)std::min<long long>((n + 255) / 256, 4ll * device_sms());
    region_stats_kernel<<<grid, 256, 0, st>>>(nv, status, n, out);
}

void launch_rehash(const RegionsDev &reg, long long n, const HashDev &hs, int *d_err, cudaStream_t st)
{
    if (n <= 0) return;
    rehash_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(reg, n, hs, d_err);
}

} // namespace am
