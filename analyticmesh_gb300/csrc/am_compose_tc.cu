// am_compose_tc.cu -- region affine composition on the 5th-generation tensor
// cores (the mixed-precision form).
//
// Same mathematics as am_compose.cu (the reference's fill_constraints,
// backend/inc/process.h:18-193): for every region, A_{l+1} = W_l diag(s_l) A_l
// (+ b_l, + skips), C = (1 - 2 s) A.  One CTA owns a tile of regions (4
// columns each, UMMA N = 4 x regions, chosen per launch from the chunk size so
// that small frontier waves still spread over every SM) and keeps the masked
// operand X_l = diag(s_l) A_l on chip the whole way through the network, as
// bf16 terms in 128B-swizzled shared memory (MN-major, or K-major for layers
// too wide for 64-column atoms): the B operand of tcgen05.mma.  The layer
// weights are the A operand (K-major); they are pre-split and
// stored in global memory as the exact shared-memory image of their 128 x 64
// blocks, so one bulk copy (cp.async.bulk, completing on an mbarrier) stages a
// block while the tensor core works on the previous one, and the first blocks
// of the next layer land while the epilogue of this one runs.
//
// Every operand is split into three bf16 terms, x = hi + mid + lo (24
// significant bits, as fp32); a block issues the six products whose weight is
// at least 2^-16 -- hh, hm, mh, hl, lh, mm.  A two-term split leaves ~2^-17
// of every operand unrepresented, which moved vertices by ~1.5e-5 and changed
// near-degenerate walk decisions.  The tensor core's fp32 accumulation error
// grows with the number of accumulate steps into one accumulator, so the
// dominant hh product and the five small correction products accumulate in
// two separate TMEM accumulators that the epilogue adds once: fp32-level
// constraint rows.  The epilogue (sixteen warps; the warps w with equal w % 4
// share TMEM lanes 32 (w % 4).. and split the columns) reads the accumulators with
// tcgen05.ld (one TMEM lane per output unit), adds bias and skips, writes the
// sign-flipped constraint rows to HBM for the polygon kernel, and writes the
// next layer's masked operand straight back into shared memory.  The face
// plane (output layer, one row) is a 4 x K dot product per region in fp32,
// one warp per region, from the operand in shared memory.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"
#include "am_tc.h"
#include "am_umma.cuh"

namespace am {

namespace {

constexpr int kThreads = 512;
constexpr int kWaitIters = 1 << 22;
constexpr int kFaceSumBytes = kThreads * 16; // face-plane partial sums: a float4 per thread

// x = hi + mid + lo in bf16 for two values at once (round to nearest each)
__device__ __forceinline__ void split2(float a, float b, uint32_t &h, uint32_t &m, uint32_t &l)
{
    const __nv_bfloat162 hb = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(hb);
    const float ra = a - hf.x, rb = b - hf.y;
    const __nv_bfloat162 mb = __floats2bfloat162_rn(ra, rb);
    const float2 mf = __bfloat1622float2(mb);
    const __nv_bfloat162 lb = __floats2bfloat162_rn(ra - mf.x, rb - mf.y);
    h = *reinterpret_cast<const uint32_t *>(&hb);
    m = *reinterpret_cast<const uint32_t *>(&mb);
    l = *reinterpret_cast<const uint32_t *>(&lb);
}

// The masked operand X (ncols x Kp, three bf16 terms `xbytes` apart) in
// shared memory, in one of two layouts.  MN-major (64-column atoms): the
// thread that owns one K row writes 8 consecutive columns with one 16-byte
// store per term.  K-major (any multiple of 16 columns, 2-byte stores): used
// when a 64-column atom of the widest K does not fit beside the weights.
struct XOp {
    uint8_t *xs;
    size_t xbytes;
    int ncols, natoms;
    bool mn;

    __device__ __forceinline__ uint32_t off(int n, int k) const
    {
        return mn ? umma::mn_sw128_offset(n, k, natoms) : umma::sw128_offset(n, k, ncols);
    }
    // columns n0 .. n0 + 2w - 1 of row k (n0 a multiple of 2w, w = 2 or 4)
    template <int w>
    __device__ __forceinline__ void put(int n0, int k, const float *v) const
    {
        uint32_t h[w], m[w], l[w];
#pragma unroll
        for (int i = 0; i < w; ++i) split2(v[2 * i], v[2 * i + 1], h[i], m[i], l[i]);
        if (mn) {
            const uint32_t o = off(n0, k);
            if (w == 4) {
                *reinterpret_cast<uint4 *>(xs + o) = make_uint4(h[0], h[1], h[2 % w], h[3 % w]);
                *reinterpret_cast<uint4 *>(xs + xbytes + o) = make_uint4(m[0], m[1], m[2 % w], m[3 % w]);
                *reinterpret_cast<uint4 *>(xs + 2 * xbytes + o) = make_uint4(l[0], l[1], l[2 % w], l[3 % w]);
            } else {
                *reinterpret_cast<uint2 *>(xs + o) = make_uint2(h[0], h[1]);
                *reinterpret_cast<uint2 *>(xs + xbytes + o) = make_uint2(m[0], m[1]);
                *reinterpret_cast<uint2 *>(xs + 2 * xbytes + o) = make_uint2(l[0], l[1]);
            }
        } else {
#pragma unroll
            for (int i = 0; i < 2 * w; ++i) {
                const uint32_t o = off(n0 + i, k);
                const int sh = (i & 1) * 16;
                *reinterpret_cast<uint16_t *>(xs + o) = (uint16_t)(h[i >> 1] >> sh);
                *reinterpret_cast<uint16_t *>(xs + xbytes + o) = (uint16_t)(m[i >> 1] >> sh);
                *reinterpret_cast<uint16_t *>(xs + 2 * xbytes + o) = (uint16_t)(l[i >> 1] >> sh);
            }
        }
    }
    // hi + mid + lo of columns n0 .. n0 + 3 (n0 a multiple of 4) of row k
    __device__ __forceinline__ void get4(int n0, int k, float *v) const
    {
        uint32_t hw[2], mw[2], lw[2];
        if (mn) {
            const uint32_t o = off(n0, k);
            const uint2 h = *reinterpret_cast<const uint2 *>(xs + o);
            const uint2 m = *reinterpret_cast<const uint2 *>(xs + xbytes + o);
            const uint2 l = *reinterpret_cast<const uint2 *>(xs + 2 * xbytes + o);
            hw[0] = h.x, hw[1] = h.y, mw[0] = m.x, mw[1] = m.y, lw[0] = l.x, lw[1] = l.y;
        } else {
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                const uint32_t o0 = off(n0 + 2 * i, k), o1 = off(n0 + 2 * i + 1, k);
                auto pair = [&](size_t t) {
                    return (uint32_t)*reinterpret_cast<const uint16_t *>(xs + t + o0) |
                           ((uint32_t)*reinterpret_cast<const uint16_t *>(xs + t + o1) << 16);
                };
                hw[i] = pair(0), mw[i] = pair(xbytes), lw[i] = pair(2 * xbytes);
            }
        }
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&hw[i]));
            const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&mw[i]));
            const float2 c = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162 *>(&lw[i]));
            v[2 * i] = a.x + b.x + c.x;
            v[2 * i + 1] = a.y + b.y + c.y;
        }
    }
    // descriptor of term u for K block kb, K step j (16 deep) of the block
    __device__ __forceinline__ uint64_t desc(int u, int kb, int j) const
    {
        const uint32_t base = umma::smem_addr(xs) + (uint32_t)(u * xbytes);
        if (mn) {
            const uint32_t kgroup = (uint32_t)natoms * 1024u;
            return umma::desc_sw128_mn(base + (uint32_t)(kb * 8 + 2 * j) * kgroup, 1024u, kgroup);
        }
        return umma::desc_sw128(base + (uint32_t)(kb * ncols * 128 + j * 32));
    }
    __device__ __forceinline__ uint32_t idesc() const
    {
        return mn ? umma::idesc_bf16_bmn(128, ncols) : umma::idesc_bf16(128, ncols);
    }
    // descriptor steps (16-byte units of the start address field) from term
    // u to u + 1 and from K step j to j + 1: desc(u, kb, j) = desc(0, kb, 0)
    // + u * ustep() + j * jstep()
    __device__ __forceinline__ uint32_t ustep() const { return (uint32_t)(xbytes >> 4); }
    __device__ __forceinline__ uint32_t jstep() const { return mn ? (uint32_t)natoms * 128u : 2u; }
};

// X[n = 4r + c][k] = s_k(r) ? -C[r][src + k][c] : 0 for k < K, 0 up to Kp
__device__ void stage_x_from_rows(const XOp &X, const float *cons, size_t rstride, const uint32_t *keys, int W, int nreg,
                                  int src, int K, int Kp)
{
    const int R = X.ncols / 4;
    for (int q = threadIdx.x; q < R * Kp; q += kThreads) {
        const int r = q / Kp, k = q % Kp;
        float x[4] = {0.f, 0.f, 0.f, 0.f};
        if (r < nreg && k < K) {
            const int row = src + k;
            if (key_bit(keys + (size_t)r * W, row)) {
                const float4 c = ld4<float>(cons + (size_t)r * rstride + (size_t)row * 4);
                x[0] = -c.x;
                x[1] = -c.y;
                x[2] = -c.z;
                x[3] = -c.w;
            }
        }
        X.put<2>(4 * r, k, x);
    }
}

__device__ __forceinline__ int mat_blocks(const TcMat &m) { return (m.Mp / 128) * (m.Kp / 64); }
__device__ __forceinline__ bool tc_skip(const SkipDev &sk) { return sk.kind == 1 && sk.from >= 1; }

// global weight block g in the order the layers consume them: linear i's
// blocks (M tile outer, K block inner), then its skip transforms
__device__ const uint8_t *block_ptr(const NetDev &net, const TcNet &tc, int g)
{
    for (int i = 1; i <= net.n_lin - 2; ++i) {
        int nb = mat_blocks(tc.lin[i]);
        if (g < nb) return tc.lin[i].blocks + (size_t)g * kWBlockBytes;
        g -= nb;
        for (int s = 0; s < net.nskip[i]; ++s)
            if (tc_skip(net.skip[i][s])) {
                nb = mat_blocks(tc.skip[i][s]);
                if (g < nb) return tc.skip[i][s].blocks + (size_t)g * kWBlockBytes;
                g -= nb;
            }
    }
    return nullptr;
}

__device__ int total_blocks(const NetDev &net, const TcNet &tc)
{
    int n = 0;
    for (int i = 1; i <= net.n_lin - 2; ++i) {
        n += mat_blocks(tc.lin[i]);
        for (int s = 0; s < net.nskip[i]; ++s)
            if (tc_skip(net.skip[i][s])) n += mat_blocks(tc.skip[i][s]);
    }
    return n;
}

// Weight-block pipeline.  A copy warp (its lane 0) streams every weight block
// of the CTA's tiles, in the order the products consume them: block h goes
// into stage h % nstage once block h - nstage's products have completed (done
// barrier).  Thread 0 issues the products of block h once its bytes have
// landed (full barrier).  Phase parity of either barrier for block h is
// (h / nstage) & 1.  h counts on across the CTA's tiles, so the next tile's
// first blocks load during this tile's last layer and every layer's first
// blocks during the previous layer's epilogue.  (Measured on GB300: with the
// copies issued by thread 0 between its products, each block cost it a wait
// for the previous block's products before the refill, and the tensor pipe
// stood idle most of the time.)
//
// Every wait is bounded.  A wait that runs out sets the error bit kErrWait
// and the CTA's abort flag: from then on no copy and no product is issued,
// the other threads skip the epilogues, and before the CTA returns the copy
// warp waits (again bounded) for its copies in flight and thread 0 for the
// products in flight, so that nothing lands in shared memory or TMEM after
// the CTA has released them.  The host reports kErrWait as a failed run.
struct WPipe {
    uint64_t *full, *done;
    uint8_t *ws;
    int nstage, total;
    int *err;
    int per_tile;          // blocks one tile consumes; the sequence repeats per tile
    int consumed;          // (thread 0) blocks whose products were issued
    volatile int *abort;   // the CTA's abort flag (shared memory)
};

__device__ __forceinline__ bool wp_wait(WPipe &p, uint64_t *bar, uint32_t parity)
{
    if (umma::mbar_wait(bar, parity, kWaitIters)) return true;
    atomicOr(p.err, kErrWait);
    *p.abort = 1;
    return false;
}

// (the copy warp's lane 0) every weight block of the CTA's tiles, nstage
// blocks ahead of the products at most
__device__ void wp_produce(WPipe &p, const NetDev &net, const TcNet &tc)
{
    int last[4] = {-1, -1, -1, -1}; // the last block copied into each stage
    for (int h = 0; h < p.total; ++h) {
        const int s = h % p.nstage;
        if (*p.abort) break;
        if (h >= p.nstage && !wp_wait(p, p.done + s, (uint32_t)((h - p.nstage) / p.nstage) & 1u)) break;
        umma::mbar_expect_tx(p.full + s, (uint32_t)kWBlockBytes);
        umma::bulk_g2s(p.ws + (size_t)s * kWBlockBytes, block_ptr(net, tc, h % p.per_tile), (uint32_t)kWBlockBytes,
                       p.full + s);
        last[s] = h;
    }
    // nothing lands in shared memory after the CTA has left (bounded)
    for (int s = 0; s < p.nstage; ++s)
        if (last[s] >= 0) umma::mbar_wait(p.full + s, (uint32_t)(last[s] / p.nstage) & 1u, kWaitIters);
}

// (thread 0) D[mt] (+)= M . X over all K blocks of the operand in shared
// memory: six products per K step (terms t, u of weight 2^-8(t+u), t + u <= 2)
__device__ void gemm_issue(WPipe &p, const TcMat &m, int mtiles, const XOp &X, uint32_t tmem, bool first, int &g)
{
    const int ncols = X.ncols;
    const uint32_t idesc = X.idesc();
    const uint64_t xu = X.ustep(), xj = X.jstep();
    const int kblocks = m.Kp / 64;
    for (int mt = 0; mt < mtiles; ++mt) {
        for (int kb = 0; kb < kblocks; ++kb) {
            if (*p.abort) return;
            const int s = g % p.nstage;
            if (!wp_wait(p, p.full + s, (uint32_t)(g / p.nstage) & 1u)) return;
            umma::fence_after();
            const uint32_t a0 = umma::smem_addr(p.ws + (size_t)s * kWBlockBytes);
            const uint32_t d_main = tmem + (uint32_t)(mt * ncols);            // hh
            const uint32_t d_corr = tmem + (uint32_t)((mtiles + mt) * ncols); // the rest
            const bool fresh = first && kb == 0;
            // A: term t at +16 KB (1024 units), K step j at +32 B (2 units)
            const uint64_t ad = umma::desc_sw128(a0), xd = X.desc(0, kb, 0);
            #pragma unroll
            for (int j = 0; j < 4; ++j) {
                umma::mma_bf16(d_main, ad + 2u * j, xd + xj * j, idesc, (fresh && j == 0) ? 0u : 1u);
                int q = 0;
                #pragma unroll
                for (int t = 0; t < 3; ++t)
                    #pragma unroll
                    for (int u = 0; u + t < 3; ++u) {
                        if (t == 0 && u == 0) continue;
                        umma::mma_bf16(d_corr, ad + 1024u * t + 2u * j, xd + xu * u + xj * j, idesc,
                                       (fresh && j == 0 && q == 0) ? 0u : 1u);
                        ++q;
                    }
            }
            umma::commit(umma::smem_addr(p.done + s)); // frees the stage for the copy warp
            p.consumed = g + 1;
            ++g;
        }
    }
}

// (thread 0) after the last block of a layer: wait until its products are in TMEM
__device__ void gemm_finish(WPipe &p, int g)
{
    if (*p.abort) return;
    const int last = g - 1;
    if (!wp_wait(p, p.done + last % p.nstage, (uint32_t)(last / p.nstage) & 1u)) return;
    umma::fence_before();
}

// (every thread, after the block barrier that follows gemm_finish) observe
// the same completion before reading the accumulators
__device__ __forceinline__ void gemm_observe(const WPipe &p, int last)
{
    if (!umma::mbar_wait(p.done + last % p.nstage, (uint32_t)(last / p.nstage) & 1u, kWaitIters)) atomicOr(p.err, kErrWait);
    umma::fence_after();
}

// (thread 0, aborting CTA) wait, bounded, for the products of the last
// committed block
__device__ void wp_drain(WPipe &p)
{
    if (p.consumed > 0)
        umma::mbar_wait(p.done + (p.consumed - 1) % p.nstage, (uint32_t)((p.consumed - 1) / p.nstage) & 1u, kWaitIters);
}

// the 512 threads of the resident tile (not the copy warp)
__device__ __forceinline__ void bar_main() { asm volatile("bar.sync 2, %0;" ::"r"(kThreads) : "memory"); }

// words between two regions' keys in shared memory: odd, so that lanes
// reading consecutive regions' bits hit distinct banks
__host__ __device__ __forceinline__ int key_stride(int W) { return W | 1; }

// tile width for a wave of `count` regions: one tile per resident slot
// while the wave is small, the widest tile otherwise
__host__ __device__ __forceinline__ int tile_cols(int count, int slots, int ncols_max)
{
    const int per = (count + slots - 1) / slots;
    const int ncols = (4 * per + 15) / 16 * 16;
    return ncols < 16 ? 16 : (ncols > ncols_max ? ncols_max : ncols);
}

__global__ void __launch_bounds__(kThreads + 32, 1) compose_tc_kernel(NetDev net, TcNet tc, RegionsDev reg, ChunkDev ch,
                                                                  float iso, int slots, int *err)
{
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t bars[4];
    __shared__ uint32_t tslot;
    __shared__ int s_last;
    __shared__ int s_abort; // a pipeline wait ran out (thread 0 or the copy warp)
    __shared__ int s_stop;  // thread 0's view of it, published before a tile barrier: uniform
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    long long head;
    int count;
    chunk_range(ch, head, count);
    if (count <= 0) return;
    const int ncols = tile_cols(count, slots, tc.ncols_max);
    const int R = ncols / 4;
    const int ntiles = (count + R - 1) / R;
    const int mytiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (mytiles == 0) return;
    int tmem_cols = 32;
    while (tmem_cols < 2 * tc.mtiles_max * ncols) tmem_cols <<= 1;
    const size_t rstride = (size_t)net.ALLP * 4;
    const int KW = key_stride(net.W); // odd: lanes on consecutive regions read distinct banks

    uint8_t *base = smem_raw + ((1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u);
    XOp X;
    X.mn = tc.mn != 0;
    X.ncols = ncols;
    X.natoms = (ncols + 63) / 64;
    X.xbytes = (size_t)(X.mn ? X.natoms * 64 : ncols) * tc.kp_max * 2; // one bf16 term of the operand
    X.xs = base;                                                     // hi, mid, lo
    uint8_t *ws = base + 3 * X.xbytes;                               // nstage weight blocks
    uint32_t *keys = reinterpret_cast<uint32_t *>(ws + (size_t)tc.nstage * kWBlockBytes); // the tile's bits
    // per CTA, for every tile: linear 0 as (w0, w1, w2, b) per unit and the
    // face-plane weights (the output linear's only row)
    float4 *w0s = reinterpret_cast<float4 *>(keys + (size_t)(tc.ncols_max / 4) * key_stride(net.W));
    float *wls = reinterpret_cast<float *>(w0s + net.nodes[1]);
    float *fsum = reinterpret_cast<float *>(reinterpret_cast<uintptr_t>(wls + net.nodes[net.n_lin - 1] + 3) & ~(uintptr_t)15);

    WPipe pp{bars, bars + 2, ws, tc.nstage, 0, err, 1, 0, &s_abort};
    pp.per_tile = total_blocks(net, tc);
    pp.total = pp.per_tile * mytiles;
    if (tid == 0) {
        s_abort = 0;
        s_stop = 0;
        for (int b = 0; b < 4; ++b) umma::mbar_init(bars + b, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) umma::tmem_alloc(&tslot, (uint32_t)tmem_cols);
    {
        const float *W0 = (const float *)net.W0;
        const float *b0 = (const float *)net.bias[0];
        for (int m = tid; tid < kThreads && m < net.nodes[1]; m += kThreads)
            w0s[m] = make_float4(W0[3 * m], W0[3 * m + 1], W0[3 * m + 2], b0[m]);
        const int il = net.n_lin - 1;
        const float *wl = (const float *)net.Wt[il]; // [K][Mp], column 0
        for (int k = tid; tid < kThreads && k < net.nodes[il]; k += kThreads) wls[k] = wl[(size_t)k * net.Mp[il]];
    }
    __syncthreads(); // barriers initialised, for the copy warp too
    if (warp == kThreads / 32) { // the copy warp: the weight blocks of every tile
        if (lane == 0) wp_produce(pp, net, tc);
        __syncwarp();
        __syncthreads(); // the tile threads' last barrier
        return;
    }
    int g = 0; // next weight block (thread 0)
    // epilogue: warp w reads TMEM lanes 32 (w % 4).. and every (kThreads / 128)-th column block
    const int q4 = warp & 3, cgrp = warp >> 2, ngrp = kThreads / 128;

    for (int j = 0; j < mytiles; ++j) {
        const long long rl0 = (long long)(blockIdx.x + (long long)j * gridDim.x) * R;
        const int nreg = (int)min((long long)R, (long long)count - rl0);
        float *cons = (float *)ch.cons + (size_t)rl0 * rstride;
        const uint32_t *gkeys = reg.keys + (size_t)(head + rl0) * net.W;
        bar_main(); // the previous tile is done with the keys and the operand
        for (int q = tid; q < R * net.W; q += kThreads)
            keys[(q / net.W) * KW + q % net.W] = q < nreg * net.W ? gkeys[q] : 0u;
        bar_main(); // every thread reads every region's bits below

        // hidden layer 1 = linear 0 rows (sign-flipped) and the extra constraints
        {
            const int n1 = net.nodes[1];
            for (int q = tid; q < nreg * n1; q += kThreads) {
                const int rr = q / n1, m = q % n1;
                const float sg = key_bit(keys + (size_t)rr * KW, m) ? -1.f : 1.f;
                const float4 w = w0s[m];
                st4<float>(cons + (size_t)rr * rstride + (size_t)m * 4, make_float4(sg * w.x, sg * w.y, sg * w.z, sg * w.w));
            }
            const float *we = (const float *)net.w_extra;
            const float *be = (const float *)net.b_extra;
            for (int q = tid; q < nreg * net.E; q += kThreads) {
                const int rr = q / net.E, e = q % net.E;
                st4<float>(cons + (size_t)rr * rstride + (size_t)(net.N + e) * 4,
                           make_float4(we[3 * e], we[3 * e + 1], we[3 * e + 2], be[e]));
            }
            // X_1 = diag(s_1) [W0 | b0]; regions fastest across the lanes:
            // consecutive regions' columns share a 128-byte operand row
            const int Kp = (n1 + 63) / 64 * 64;
            for (int q = tid; q < R * Kp; q += kThreads) {
                const int r = q % R, k = q / R;
                float x[4] = {0.f, 0.f, 0.f, 0.f};
                if (r < nreg && k < n1 && key_bit(keys + (size_t)r * KW, k)) {
                    const float4 w = w0s[k];
                    x[0] = w.x;
                    x[1] = w.y;
                    x[2] = w.z;
                    x[3] = w.w;
                }
                X.put<2>(4 * r, k, x);
            }
        }
        umma::fence_proxy_async();
        umma::fence_before();
        bar_main();
        umma::fence_after();
        const uint32_t tmem = tslot;

        for (int i = 1; i <= net.n_lin - 2; ++i) {
            const int M = net.nodes[i + 1];
            const int mtiles = (M + 127) / 128;
            if (tid == 0) gemm_issue(pp, tc.lin[i], mtiles, X, tmem, true, g);
            for (int s = 0; s < net.nskip[i]; ++s) {
                const SkipDev &sk = net.skip[i][s];
                if (tc_skip(sk)) {
                    // the operand is about to be overwritten: the products so far must be done
                    if (tid == 0) {
                        gemm_finish(pp, g);
                        if (*pp.abort) s_stop = 1;
                    }
                    bar_main();
                    if (s_stop) break; // written by thread 0 before the barrier: uniform
                    stage_x_from_rows(X, cons, rstride, keys, KW, nreg, net.hoff[sk.from],
                                      net.nodes[sk.from], tc.skip[i][s].Kp);
                    umma::fence_proxy_async();
                    bar_main();
                    if (tid == 0) gemm_issue(pp, tc.skip[i][s], mtiles, X, tmem, false, g);
                }
            }
            // the first M tile's bias, loaded while the products run
            const float *bias = (const float *)net.bias[i];
            float bnext = q4 * 32 + lane < M ? bias[q4 * 32 + lane] : 0.f;
            if (tid == 0) {
                gemm_finish(pp, g);
                if (*pp.abort) s_stop = 1;
                s_last = g - 1;
            }
            __syncwarp();
            bar_main();
            if (s_stop) break; // no epilogue: the accumulators are not complete
            gemm_observe(pp, s_last);
            // epilogue: accumulators -> constraint rows (HBM) and the next operand (smem)
            const int Kn = (M + 63) / 64 * 64; // next operand's padded K (the face plane reads it too)
            for (int q = tid; q < R * (Kn - M); q += kThreads) {
                const int r = q % R, k = M + q / R;
                const float z[4] = {0.f, 0.f, 0.f, 0.f};
                X.put<2>(4 * r, k, z);
            }
            for (int mt = 0; mt < mtiles; ++mt) {
                const int m = mt * 128 + q4 * 32 + lane;
                const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
                const float bm = bnext;
                if (mt + 1 < mtiles) bnext = m + 128 < M ? bias[m + 128] : 0.f;
                const int row = net.hoff[i + 1] + m;
                for (int cb = cgrp; cb < ncols / 16; cb += ngrp) {
                    float v[16], vc[16];
                    umma::tmem_ld16x2(lane_base + (uint32_t)(mt * ncols + cb * 16),
                                      lane_base + (uint32_t)((mtiles + mt) * ncols + cb * 16), v, vc);
                    if (m >= M) continue;
                    float x[16]; // next operand, columns cb * 16 .. + 15 of row k = m
                    #pragma unroll
                    for (int qq = 0; qq < 4; ++qq) {
                        const int r = cb * 4 + qq;
                        x[4 * qq] = x[4 * qq + 1] = x[4 * qq + 2] = x[4 * qq + 3] = 0.f;
                        if (r < nreg) {
                            const uint32_t *key = keys + (size_t)r * KW;
                            float *cr = cons + (size_t)r * rstride;
                            float o[4] = {v[4 * qq] + vc[4 * qq], v[4 * qq + 1] + vc[4 * qq + 1],
                                          v[4 * qq + 2] + vc[4 * qq + 2], v[4 * qq + 3] + vc[4 * qq + 3] + bm};
                            for (int s = 0; s < net.nskip[i]; ++s) {
                                const SkipDev &sk = net.skip[i][s];
                                if (sk.kind == 0) {
                                    if (sk.from == 0) {
                                        if (m < 3) o[m] += 1.f;
                                    } else {
                                        const int srow = net.hoff[sk.from] + m;
                                        if (key_bit(key, srow)) {
                                            const float4 c = ld4<float>(cr + (size_t)srow * 4);
                                            o[0] -= c.x;
                                            o[1] -= c.y;
                                            o[2] -= c.z;
                                            o[3] -= c.w;
                                        }
                                    }
                                } else if (sk.from == 0) {
                                    const float *tt = (const float *)sk.tmt;
                                    o[0] += tt[m];
                                    o[1] += tt[(size_t)sk.Mp + m];
                                    o[2] += tt[2 * (size_t)sk.Mp + m];
                                }
                            }
                            const bool act = key_bit(key, row);
                            const float sg = act ? -1.f : 1.f;
                            st4<float>(cr + (size_t)row * 4, make_float4(sg * o[0], sg * o[1], sg * o[2], sg * o[3]));
                            if (act) {
                                x[4 * qq] = o[0];
                                x[4 * qq + 1] = o[1];
                                x[4 * qq + 2] = o[2];
                                x[4 * qq + 3] = o[3];
                            }
                        }
                    }
                    X.put<4>(cb * 16, m, x);
                    X.put<4>(cb * 16 + 8, m, x + 8);
                }
            }
            umma::fence_proxy_async();
            umma::fence_before();
            bar_main();
            umma::fence_after();
        }

        if (s_stop) break;
        // face plane: w_eq = W_L . X_L (+ b_L, + connections into the output layer)
        // in fp32 from the operand in shared memory (hi + mid + lo is exact):
        // lanes take regions (consecutive regions share operand rows), the
        // warps split K, partial sums meet in shared memory
        {
            const int i = net.n_lin - 1;
            const int K = net.nodes[i];
            const float bl = ((const float *)net.bias[i])[0];
            constexpr int kWarps = kThreads / 32;
            for (int r0 = 0; r0 < R; r0 += 32) {
                const int r = r0 + lane;
                float acc[4] = {0.f, 0.f, 0.f, 0.f};
                if (r < R)
                    for (int k = warp; k < K; k += kWarps) {
                        const float w = wls[k];
                        float x[4];
                        X.get4(4 * r, k, x);
#pragma unroll
                        for (int c = 0; c < 4; ++c) acc[c] = fmaf(w, x[c], acc[c]);
                    }
                // partial sums: [warp][lane][4]
                reinterpret_cast<float4 *>(fsum)[warp * 32 + lane] = make_float4(acc[0], acc[1], acc[2], acc[3]);
                bar_main();
                if (tid < 128) {
                    const int rr = tid >> 2, c = tid & 3, rg = r0 + rr;
                    float a = 0.f;
                    for (int w = 0; w < kWarps; ++w) a += fsum[(w * 32 + rr) * 4 + c];
                    if (rg < nreg) {
                        const uint32_t *key = keys + (size_t)rg * KW;
                        const float *cr = cons + (size_t)rg * rstride;
                        for (int s = 0; s < net.nskip[i]; ++s) {
                            const SkipDev &sk = net.skip[i][s];
                            if (sk.kind == 0) {
                                if (sk.from >= 1 && net.nodes[sk.from] == 1 && key_bit(key, net.hoff[sk.from]))
                                    a -= cr[(size_t)net.hoff[sk.from] * 4 + c];
                            } else if (sk.from == 0) {
                                if (c < 3) a += ((const float *)sk.tmt)[(size_t)c * sk.Mp];
                            } else {
                                const float *tt = (const float *)sk.tmt; // [dec][Mp]
                                const int hs = net.hoff[sk.from];
                                for (int k = 0; k < net.nodes[sk.from]; ++k)
                                    if (key_bit(key, hs + k)) a -= tt[(size_t)k * sk.Mp] * cr[(size_t)(hs + k) * 4 + c];
                            }
                        }
                        if (c == 3) a += bl - iso;
                        ((float *)ch.eq)[(size_t)(rl0 + rg) * 4 + c] = a;
                    }
                }
                bar_main();
            }
        }
    } // tiles
    if (tid == 0 && *pp.abort) wp_drain(pp);
    umma::fence_before();
    __syncthreads(); // with the copy warp
    if (warp == 0) umma::tmem_dealloc(tslot, (uint32_t)tmem_cols);
}

// ---------------------------------------------------------------- streamed operand
// Wide layers: three bf16 terms of a resident K x ncols operand leave room for
// only a few regions per tile, and every tile streams all weight blocks again.
// Here the operand is not resident.  The epilogue writes the constraint rows
// only; the next layer's masked operand is rebuilt one 64-deep K block at a
// time from those rows (just written, still in L2) into a two-stage ring by
// sixteen builder warps while one issuing thread runs the products on the
// other stage.  K blocks are the outer loop of the products, so one block of
// the operand serves every M tile of the layer and the tile is as wide as
// TMEM allows (two accumulators per M tile in 512 columns).  The operand
// values, the order of the products into each accumulator and the epilogue
// and face-plane arithmetic are those of compose_tc_kernel, so both kernels
// give the same bits.
constexpr int kSBuild = 512;            // builder threads (16 warps)
constexpr int kSThreads = kSBuild + 64; // + the issuing warp and the weight-copy warp
constexpr int kSFaceSumBytes = kSBuild * 16;

__device__ __forceinline__ int jobs_of(const NetDev &net, int i)
{
    int n = 1;
    for (int s = 0; s < net.nskip[i]; ++s) n += tc_skip(net.skip[i][s]) ? 1 : 0;
    return n;
}

// product job `job` of linear i: 0 = the linear itself on hidden layer i,
// q >= 1 = its q-th tensor-core connection (a transform of an earlier layer)
__device__ const TcMat &job_mat(const NetDev &net, const TcNet &tc, int i, int job, int &src)
{
    src = i;
    if (job > 0) {
        int q = 0;
        for (int s = 0; s < net.nskip[i]; ++s)
            if (tc_skip(net.skip[i][s]) && ++q == job) {
                src = net.skip[i][s].from;
                return tc.skip[i][s];
            }
    }
    return tc.lin[i];
}

__device__ __forceinline__ void bar_builders() { asm volatile("bar.sync 1, %0;" ::"r"(kSBuild) : "memory"); }

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(umma::smem_addr(bar)) : "memory");
}

// Bounded wait of the streamed kernel: false at once when the CTA is
// aborting, and false -- with the error bit kErrWait and the abort flag set --
// when the wait runs out.  An aborting CTA keeps its arrive / commit / barrier
// sequence (so that no thread waits on a partner that gave up) but issues no
// copy or product and skips the epilogue work.
__device__ __forceinline__ bool swait(uint64_t *bar, uint32_t parity, int *err, volatile int *abort)
{
    // the phase test and the abort flag's load overlap (the issuing
    // thread's critical path between two blocks of products)
    const bool ready = umma::mbar_test(bar, parity);
    const int ab = *abort;
    if (ab) return false;
    if (ready || umma::mbar_wait(bar, parity, kWaitIters)) return true;
    atomicOr(err, kErrWait);
    *abort = 1;
    return false;
}

// (one thread of its own warp) the weight blocks through the nstage ring, in
// the order the products consume them -- tile, layer, job, K block, M tile --
// running ahead of the products by up to nstage blocks: block h goes into
// stage h % nstage once the products of block h - nstage have completed.
// Measured on GB300: with the copies issued from the same thread as the
// products, every block cost that thread a wait for the previous block's
// products before its refill (about as long as the 24 products themselves),
// so the tensor pipe was idle most of the time.
__device__ void produce_streamed(const NetDev &net, const TcNet &tc, uint8_t *ws, uint64_t *wfull, uint64_t *wdone,
                                 int tiles, int *err, volatile int *abort)
{
    const int nst = tc.nstage;
    int h = 0;
    int ps = 0;        // stage of block h (h % nst) ...
    uint32_t pph = 0u; // ... and (h / nst) & 1, kept incrementally
    int last[4] = {-1, -1, -1, -1}; // the last block copied into each stage
    for (int t = 0; t < tiles; ++t)
        for (int i = 1; i <= net.n_lin - 2; ++i) {
            const int mtl = (net.nodes[i + 1] + 127) / 128, mper = (mtl + tc.mgroups - 1) / tc.mgroups;
            for (int mt0 = 0; mt0 < mtl; mt0 += mper) {
            const int njobs = jobs_of(net, i);
            for (int job = 0; job < njobs; ++job) {
                int src;
                const TcMat &m = job_mat(net, tc, i, job, src);
                const int mtiles = m.Mp / 128, kblocks = m.Kp / 64;
                for (int kb = 0; kb < kblocks; ++kb)
                    for (int mt = mt0; mt < min(mtiles, mt0 + mper); ++mt, ++h) {
                        const int s = ps;
                        const uint32_t ph = pph; // phase of block h - nst's products
                        if (++ps == nst) {
                            ps = 0;
                            pph ^= 1u;
                        }
                        if (h >= nst && !swait(wdone + s, ph ^ 1u, err, abort)) continue;
                        if (*abort) continue;
                        umma::mbar_expect_tx(wfull + s, (uint32_t)kWBlockBytes);
                        umma::bulk_g2s(ws + (size_t)s * kWBlockBytes,
                                       m.blocks + (size_t)(mt * kblocks + kb) * kWBlockBytes, (uint32_t)kWBlockBytes,
                                       wfull + s);
                        last[s] = h;
                    }
            }
            }
        }
    // nothing lands in shared memory after the CTA has left: the last copy of
    // every stage (bounded)
    for (int s = 0; s < nst; ++s)
        if (last[s] >= 0) umma::mbar_wait(wfull + s, (uint32_t)(last[s] / nst) & 1u, kWaitIters);
}

// (one thread) the products: operand blocks through the two-stage ring,
// weight blocks from the producer's ring, six products per K step into the
// main (hi.hi) and the correction accumulator of each M tile.  The commits
// that free the operand stages and publish the layer's accumulators are
// made whatever happens, so that the builders never wait on a partner that
// gave up.
__device__ void issue_streamed(const NetDev &net, const TcNet &tc, uint8_t *ws, uint64_t *wfull, uint64_t *wdone,
                               const XOp *XS, uint64_t *xfull, uint64_t *xdone, uint64_t *accdone, uint32_t tmem,
                               int ncols, int tiles, int *err, volatile int *abort)
{
    const int nst = tc.nstage;
    int h = 0, xb = 0, consumed = 0;
    int ws_ = 0;       // stage of weight block h (h % nst) ...
    uint32_t wph = 0u; // ... and its phase parity ((h / nst) & 1), kept incrementally
    // weight stage q's descriptor = wd0 + q * wstep (start address field)
    const uint64_t wd0 = umma::desc_sw128(umma::smem_addr(ws));
    const uint64_t wstep = (uint64_t)(kWBlockBytes >> 4);
    // operand descriptors of the two stages; term and K step add constant offsets
    const uint64_t xd0 = XS[0].desc(0, 0, 0), xd1 = XS[1].desc(0, 0, 0);
    const uint64_t xu = XS[0].ustep(), xj = XS[0].jstep();
    const uint32_t idesc = XS[0].idesc();
    for (int t = 0; t < tiles; ++t)
        for (int i = 1; i <= net.n_lin - 2; ++i) {
            const int mtl = (net.nodes[i + 1] + 127) / 128, mper = (mtl + tc.mgroups - 1) / tc.mgroups;
            for (int mt0 = 0; mt0 < mtl; mt0 += mper) { // a group of M tiles, its own accumulators
            const int njobs = jobs_of(net, i);
            for (int job = 0; job < njobs; ++job) {
                int src;
                const TcMat &m = job_mat(net, tc, i, job, src);
                const int mtiles = m.Mp / 128, kblocks = m.Kp / 64;
                for (int kb = 0; kb < kblocks; ++kb) {
                    const int xs = xb & 1;
                    const uint64_t xd = xs ? xd1 : xd0;
                    const bool xok = swait(xfull + xs, (uint32_t)(xb >> 1) & 1u, err, abort); // operand block built
                    const bool fresh = job == 0 && kb == 0;
                    for (int mt = mt0; mt < min(mtiles, mt0 + mper); ++mt, ++h) {
                        const int s = ws_;
                        const uint32_t ph = wph;
                        if (++ws_ == nst) {
                            ws_ = 0;
                            wph ^= 1u;
                        }
                        if (!xok || !swait(wfull + s, ph, err, abort)) continue;
                        umma::fence_after();
                        const uint32_t d_main = tmem + (uint32_t)((mt - mt0) * ncols);
                        const uint32_t d_corr = tmem + (uint32_t)((mper + mt - mt0) * ncols);
                        const uint64_t ad = wd0 + wstep * (uint64_t)s; // term t at +16 KB, K step j at +32 B
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            umma::mma_bf16(d_main, ad + 2u * j, xd + xj * j, idesc, (fresh && j == 0) ? 0u : 1u);
                            int q = 0;
#pragma unroll
                            for (int tt = 0; tt < 3; ++tt)
#pragma unroll
                                for (int u = 0; u + tt < 3; ++u) {
                                    if (tt == 0 && u == 0) continue;
                                    umma::mma_bf16(d_corr, ad + 1024u * tt + 2u * j, xd + xu * u + xj * j, idesc,
                                                   (fresh && j == 0 && q == 0) ? 0u : 1u);
                                    ++q;
                                }
                        }
                        umma::commit(umma::smem_addr(wdone + s)); // the producer may refill the stage
                        consumed = h + 1;
                    }
                    umma::commit(umma::smem_addr(xdone + xs)); // the operand stage is free once these complete
                    ++xb;
                }
            }
            umma::commit(umma::smem_addr(accdone)); // the group's accumulators are complete
            }
        }
    // the last products have completed before TMEM is released
    if (consumed > 0 &&
        !umma::mbar_wait(wdone + (consumed - 1) % nst, (uint32_t)((consumed - 1) / nst) & 1u, kWaitIters))
        atomicOr(err, kErrWait);
}

__global__ void __launch_bounds__(kSThreads, 1) compose_tcs_kernel(NetDev net, TcNet tc, RegionsDev reg, ChunkDev ch,
                                                                    float iso, int slots, int *err)
{
    extern __shared__ uint8_t smem_raw[];
    // wfull[3], wdone[3] (weight ring), xfull[2], xdone[2] (operand ring), accdone
    __shared__ uint64_t bars[11];
    __shared__ uint32_t tslot;
    __shared__ int s_abort; // a wait ran out: nothing more is issued, epilogues are skipped
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    long long head;
    int count;
    chunk_range(ch, head, count);
    if (count <= 0) return;
    const int ncols = tile_cols(count, slots, tc.ncols_max);
    const int R = ncols / 4;
    const int ntiles = (count + R - 1) / R;
    const int tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    if (tiles == 0) return;
    int tmem_cols = 32;
    const int mper_max = (tc.mtiles_max + tc.mgroups - 1) / tc.mgroups;
    while (tmem_cols < 2 * mper_max * ncols) tmem_cols <<= 1;
    const size_t rstride = (size_t)net.ALLP * 4;
    const int KW = key_stride(net.W); // odd: lanes on consecutive regions read distinct banks

    uint8_t *base = smem_raw + ((1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u);
    XOp XS[2];
    const int natoms = (ncols + 63) / 64;
    const size_t plane = (size_t)(tc.mn ? natoms * 64 : ncols) * 64 * 2; // one term of one K block
    for (int x = 0; x < 2; ++x) {
        XS[x].mn = tc.mn != 0;
        XS[x].ncols = ncols;
        XS[x].natoms = natoms;
        XS[x].xbytes = plane;
        XS[x].xs = base + (size_t)x * 3 * plane; // hi, mid, lo
    }
    uint8_t *ws = base + 6 * plane;
    uint32_t *keys = reinterpret_cast<uint32_t *>(ws + (size_t)tc.nstage * kWBlockBytes);
    float4 *w0s = reinterpret_cast<float4 *>(keys + (size_t)(tc.ncols_max / 4) * key_stride(net.W));
    float *wls = reinterpret_cast<float *>(w0s + net.nodes[1]);
    // the face plane's partial sums use the operand ring: it is idle then
    // (the tile's products are complete, the next tile's operand not begun)
    float *fsum = reinterpret_cast<float *>(base);
    uint64_t *wfull = bars, *wdone = bars + 3, *xfull = bars + 6, *xdone = bars + 8, *accdone = bars + 10;

    volatile int *abort = &s_abort;
    if (tid == 0) {
        s_abort = 0;
        for (int b = 0; b < 6; ++b) umma::mbar_init(bars + b, 1);
        umma::mbar_init(xfull, kSBuild);
        umma::mbar_init(xfull + 1, kSBuild);
        umma::mbar_init(xdone, 1);
        umma::mbar_init(xdone + 1, 1);
        umma::mbar_init(accdone, 1);
        umma::fence_mbar_init();
    }
    if (warp == 0) umma::tmem_alloc(&tslot, (uint32_t)tmem_cols);
    {
        const float *W0 = (const float *)net.W0;
        const float *b0 = (const float *)net.bias[0];
        for (int m = tid; m < net.nodes[1]; m += kSThreads)
            w0s[m] = make_float4(W0[3 * m], W0[3 * m + 1], W0[3 * m + 2], b0[m]);
        const int il = net.n_lin - 1;
        const float *wl = (const float *)net.Wt[il]; // [K][Mp], column 0
        for (int k = tid; k < net.nodes[il]; k += kSThreads) wls[k] = wl[(size_t)k * net.Mp[il]];
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;

    if (warp == kSBuild / 32) {
        if (lane == 0)
            issue_streamed(net, tc, ws, wfull, wdone, XS, xfull, xdone, accdone, tmem, ncols, tiles, err, abort);
        __syncwarp(); // the warp reaches the block barrier below converged
    } else if (warp == kSBuild / 32 + 1) {
        if (lane == 0) produce_streamed(net, tc, ws, wfull, wdone, tiles, err, abort);
        __syncwarp();
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4).. and every fourth column block
        const int q4 = warp & 3, cgrp = warp >> 2, ngrp = kSBuild / 128;
        int xb = 0, accph = 0;
        for (int j = 0; j < tiles; ++j) {
            const long long rl0 = (long long)(blockIdx.x + (long long)j * gridDim.x) * R;
            const int nreg = (int)min((long long)R, (long long)count - rl0);
            float *cons = (float *)ch.cons + (size_t)rl0 * rstride;
            const uint32_t *gkeys = reg.keys + (size_t)(head + rl0) * net.W;
            bar_builders(); // the previous tile is done with the keys
            for (int q = tid; q < R * net.W; q += kSBuild)
                keys[(q / net.W) * KW + q % net.W] = q < nreg * net.W ? gkeys[q] : 0u;
            bar_builders();
            // hidden layer 1 = linear 0 rows (sign-flipped) and the extra constraints
            const int n1 = net.nodes[1];
            for (int q = tid; q < nreg * n1; q += kSBuild) {
                const int rr = q / n1, m = q % n1;
                const float sg = key_bit(keys + (size_t)rr * KW, m) ? -1.f : 1.f;
                const float4 w = w0s[m];
                st4<float>(cons + (size_t)rr * rstride + (size_t)m * 4, make_float4(sg * w.x, sg * w.y, sg * w.z, sg * w.w));
            }
            const float *we = (const float *)net.w_extra;
            const float *be = (const float *)net.b_extra;
            for (int q = tid; q < nreg * net.E; q += kSBuild) {
                const int rr = q / net.E, e = q % net.E;
                st4<float>(cons + (size_t)rr * rstride + (size_t)(net.N + e) * 4,
                           make_float4(we[3 * e], we[3 * e + 1], we[3 * e + 2], be[e]));
            }
            bar_builders(); // layer-1 rows written by every builder

            // X[4r + c][k] = s_k(r) ? -C[r][k][c] : 0 (layer 1: +W0 rows from
            // shared memory), one 64-deep K block at a time; every pass of a
            // layer streams the same blocks.  Thread tid owns the items q = tid
            // + u kSBuild (region q % R, row q / R of the block): regions
            // fastest across the lanes.  The first four items of the next
            // block are loaded one step ahead, so that their latency hides
            // behind the stage wait; raw values are kept and signed when
            // stored.
            auto load_items = [&](int li, int job, int kb, int c, float4 *v) {
                int src;
                job_mat(net, tc, li, job, src);
                const int K = net.nodes[src], rows0 = net.hoff[src];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int q = tid + (4 * c + u) * kSBuild;
                    const int r = q % R, k = kb * 64 + q / R;
                    float4 x = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (q < R * 64 && r < nreg && k < K && key_bit(keys + (size_t)r * KW, rows0 + k))
                        x = src == 1 ? w0s[k] : ld4<float>(cons + (size_t)r * rstride + (size_t)(rows0 + k) * 4);
                    v[u] = x;
                }
            };
            auto put_items = [&](const XOp &X, int c, const float4 *v, float sg) {
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int q = tid + (4 * c + u) * kSBuild;
                    if (q < R * 64) {
                        const float x[4] = {sg * v[u].x, sg * v[u].y, sg * v[u].z, sg * v[u].w};
                        X.put<2>(4 * (q % R), q / R, x);
                    }
                }
            };
            const int nchunks = (R * 64 + 4 * kSBuild - 1) / (4 * kSBuild);
            // The epilogue of a pass reads its accumulators (warp w: TMEM
            // lanes 32 (w % 4).., column blocks cgrp, cgrp + ngrp, ... of each
            // M tile; at most four blocks of 16 columns) and stores their rows,
            // except the last block, which stays in registers and is stored
            // during the next pass's first step, while the tensor core works
            // (a pass's 128 KB of rows take ~4 K cycles of the SM's store
            // bandwidth alone, measured on GB300; registers allow one block).
            // A barrier follows the deferred store, so that later loads see
            // the rows.
            const int ncb = ncols / 16;
            const int ncbw = cgrp < ncb ? (ncb - cgrp + ngrp - 1) / ngrp : 0; // this warp's column blocks
            const int ncbu = (ncb + ngrp - 1) / ngrp;                          // the most any warp has
            const uint32_t lane_base = tmem + ((uint32_t)(q4 * 32) << 16);
            // o[0..kKeep-1][16]: the (at most kKeep) deferred column blocks in
            // store order -- the first blocks of a pass are stored at once,
            // before the TMEM is given up; a stored block leaves o[0] and the
            // others move up (constant indices only, so that the blocks stay
            // in registers; more than one block spilled at 96 registers)
            constexpr int kKeep = 1;
            float o[kKeep][16];
            int nd = 0, def_i = 1, def_mt0 = 0; // deferred column blocks (uniform count), their pass
            int def_first = 0, def_nit = 0;     // this warp's first deferred block, its blocks in that pass
            bool def_ok = false;
            auto shift_o = [&]() {
#pragma unroll
                for (int b = 0; b + 1 < kKeep; ++b)
#pragma unroll
                    for (int k = 0; k < 16; ++k) o[b][k] = o[b + 1][k];
            };
            auto store_block = [&](int it) { // block it of the pass def_i / def_mt0, from o[0]
                if (!def_ok || it >= def_nit) return; // (this warp's share)
                const int li = def_i;
                const int mt = def_mt0 + it / ncbw, cb = cgrp + (it % ncbw) * ngrp;
                const int m = mt * 128 + q4 * 32 + lane;
                if (m >= net.nodes[li + 1]) return;
                const int row = net.hoff[li + 1] + m;
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const int r = cb * 4 + qq;
                    if (r >= nreg) continue;
                    const uint32_t *key = keys + (size_t)r * KW;
                    float *cr = cons + (size_t)r * rstride;
                    float v4[4] = {o[0][4 * qq], o[0][4 * qq + 1], o[0][4 * qq + 2], o[0][4 * qq + 3]};
                    for (int s = 0; s < net.nskip[li]; ++s) {
                        const SkipDev &sk = net.skip[li][s];
                        if (sk.kind == 0) {
                            if (sk.from == 0) {
                                if (m < 3) v4[m] += 1.f;
                            } else {
                                const int srow = net.hoff[sk.from] + m;
                                if (key_bit(key, srow)) {
                                    const float4 c = ld4<float>(cr + (size_t)srow * 4);
                                    v4[0] -= c.x;
                                    v4[1] -= c.y;
                                    v4[2] -= c.z;
                                    v4[3] -= c.w;
                                }
                            }
                        } else if (sk.from == 0) {
                            const float *tt = (const float *)sk.tmt;
                            v4[0] += tt[m];
                            v4[1] += tt[(size_t)sk.Mp + m];
                            v4[2] += tt[2 * (size_t)sk.Mp + m];
                        }
                    }
                    const float sg = key_bit(key, row) ? -1.f : 1.f;
                    st4<float>(cr + (size_t)row * 4, make_float4(sg * v4[0], sg * v4[1], sg * v4[2], sg * v4[3]));
                }
            };
            float4 pre[4];
            for (int i = 1; i <= net.n_lin - 2; ++i) {
                const int M = net.nodes[i + 1];
                const int mtiles = (M + 127) / 128;
                const int mper = (mtiles + tc.mgroups - 1) / tc.mgroups;
                const int njobs = jobs_of(net, i);
                load_items(i, 0, 0, 0, pre);
                for (int mt0 = 0; mt0 < mtiles; mt0 += mper) { // the products of this group of M tiles
                const int mt1 = min(mtiles, mt0 + mper);
                int t = 0; // step of the pass
                for (int job = 0; job < njobs; ++job) {
                    int src;
                    const TcMat &mat = job_mat(net, tc, i, job, src);
                    const float sg = src == 1 ? 1.f : -1.f;
                    const int nkb = mat.Kp / 64;
                    for (int kb = 0; kb < nkb; ++kb, ++t) {
                        // the next block: of this pass, else the next pass's
                        // first (the next layer's first is loaded when the
                        // layer begins: registers)
                        int njob = job, nkb2 = kb + 1;
                        bool more = true;
                        if (nkb2 == nkb) {
                            nkb2 = 0;
                            if (++njob == njobs) {
                                njob = 0;
                                more = mt1 < mtiles;
                            }
                        }
                        const int xs = xb & 1, fill = xb >> 1;
                        // stage free (an aborting CTA builds nothing but still arrives)
                        const bool ok = fill < 1 ? !*abort : swait(xdone + xs, (uint32_t)((fill - 1) & 1), err, abort);
                        const XOp &X = XS[xs];
                        if (ok) {
                            put_items(X, 0, pre, sg);
                            for (int c = 1; c < nchunks; ++c) {
                                float4 t4[4];
                                load_items(i, job, kb, c, t4);
                                put_items(X, c, t4, sg);
                            }
                        }
                        umma::fence_proxy_async(); // generic-proxy stores -> the tensor cores
                        mbar_arrive(xfull + xs);
                        ++xb;
                        if (t < nd) {
                            store_block(def_first + t);
                            shift_o();
                            if (t == nd - 1) bar_builders();
                        }
                        if (more) load_items(i, njob, nkb2, 0, pre);
                    }
                }
                if (t < nd) { // a pass shorter than the deferred blocks
                    for (; t < nd; ++t) {
                        store_block(def_first + t);
                        shift_o();
                    }
                    bar_builders();
                }
                nd = 0;
                const float *bias = (const float *)net.bias[i];
                const int mA = mt0 * 128 + q4 * 32 + lane, mB = mA + 128;
                const float bA = mA < M ? bias[mA] : 0.f;                   // loaded while the products run
                const float bB = mt0 + 1 < mt1 && mB < M ? bias[mB] : 0.f;
                // the layer's products are in TMEM; the TMEM loads below are
                // warp-collective, so the warp decides as one
                bool acc_ok = swait(accdone, (uint32_t)(accph & 1), err, abort);
                acc_ok = __all_sync(0xffffffffu, acc_ok) && !__any_sync(0xffffffffu, *abort != 0);
                ++accph;
                umma::fence_after();
                // accumulators -> registers: main + correction (+ bias); the
                // first blocks are stored at once, the last two (at most)
                // kept in o for the next pass's first steps
                const int nit = (mt1 - mt0) * ncbw;
                const int nkeep = min(kKeep, nit);
                def_i = i;
                def_mt0 = mt0;
                def_ok = acc_ok;
                def_nit = nit;
                def_first = nit - nkeep;
#pragma unroll
                for (int it = 0; it < 4; ++it) {
                    if (!acc_ok || it >= nit) break;
                    const int mt = mt0 + it / ncbw, cb = cgrp + (it % ncbw) * ngrp;
                    const int mm = mt * 128 + q4 * 32 + lane;
                    const float bm = mt == mt0 ? bA : (mt == mt0 + 1 ? bB : (mm < M ? bias[mm] : 0.f));
                    // (eight columns at a time: fewer live registers; the
                    // destination block by constant index: registers)
                    const uint32_t ta = lane_base + (uint32_t)((mt - mt0) * ncols + cb * 16);
                    const uint32_t tb = lane_base + (uint32_t)((mper + mt - mt0) * ncols + cb * 16);
                    if (it < def_first) { // stored now
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float v[8], vc[8];
                            umma::tmem_ld8x2(ta + 8 * h, tb + 8 * h, v, vc);
#pragma unroll
                            for (int k = 0; k < 8; ++k) o[0][8 * h + k] = (k & 3) == 3 ? v[k] + vc[k] + bm : v[k] + vc[k];
                        }
                        store_block(it);
                    } else { // kept: into o[kKeep - 1] after the earlier kept ones moved up
                        if (kKeep > 1) shift_o();
#pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            float v[8], vc[8];
                            umma::tmem_ld8x2(ta + 8 * h, tb + 8 * h, v, vc);
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                o[kKeep - 1][8 * h + k] = (k & 3) == 3 ? v[k] + vc[k] + bm : v[k] + vc[k];
                        }
                    }
                }
                for (int b = nkeep; b < kKeep; ++b) shift_o(); // the kept blocks from o[0] on
                umma::fence_before(); // TMEM read out before the next products overwrite it
                nd = min(kKeep, (mt1 - mt0) * ncbu);
                // the kept rows: stored during the next pass of this layer,
                // or the next layer's first (whose early blocks read only rows
                // of this layer's earlier passes and of this pass's first
                // blocks ...), else now
                const bool defer = mt1 < mtiles || (i < net.n_lin - 2 && nd <= 2 * mt0);
                if (!defer) {
                    for (int t2 = 0; t2 < nd; ++t2) {
                        store_block(def_first + t2);
                        shift_o();
                    }
                    nd = 0;
                    bar_builders(); // rows of hidden layer i + 1 written by every builder
                }
                }
            }

            // face plane: w_eq = W_L . X_L, X_L = -C of the last hidden layer
            // where active; lanes take regions, the warps split K, partial
            // sums meet in shared memory (the order of compose_tc_kernel)
            {
                const int i = net.n_lin - 1;
                const int K = net.nodes[i], rows0 = net.hoff[i];
                const float bl = ((const float *)net.bias[i])[0];
                constexpr int kWarps = kSBuild / 32;
                const bool live = !*abort; // per thread: the barriers below are kept either way
                for (int r0 = 0; r0 < R; r0 += 32) {
                    const int r = r0 + lane;
                    float acc[4] = {0.f, 0.f, 0.f, 0.f};
                    if (live && r < nreg)
                        for (int k = warp; k < K; k += kWarps) {
                            const float w = wls[k];
                            float x[4] = {0.f, 0.f, 0.f, 0.f};
                            if (key_bit(keys + (size_t)r * KW, rows0 + k)) {
                                const float4 c = ld4<float>(cons + (size_t)r * rstride + (size_t)(rows0 + k) * 4);
                                x[0] = -c.x, x[1] = -c.y, x[2] = -c.z, x[3] = -c.w;
                            }
#pragma unroll
                            for (int c = 0; c < 4; ++c) acc[c] = fmaf(w, x[c], acc[c]);
                        }
                    reinterpret_cast<float4 *>(fsum)[warp * 32 + lane] = make_float4(acc[0], acc[1], acc[2], acc[3]);
                    bar_builders();
                    if (live && tid < 128) {
                        const int rr = tid >> 2, c = tid & 3, rg = r0 + rr;
                        float a = 0.f;
                        for (int w = 0; w < kWarps; ++w) a += fsum[(w * 32 + rr) * 4 + c];
                        if (rg < nreg) {
                            const uint32_t *key = keys + (size_t)rg * KW;
                            const float *cr = cons + (size_t)rg * rstride;
                            for (int s = 0; s < net.nskip[i]; ++s) {
                                const SkipDev &sk = net.skip[i][s];
                                if (sk.kind == 0) {
                                    if (sk.from >= 1 && net.nodes[sk.from] == 1 && key_bit(key, net.hoff[sk.from]))
                                        a -= cr[(size_t)net.hoff[sk.from] * 4 + c];
                                } else if (sk.from == 0) {
                                    if (c < 3) a += ((const float *)sk.tmt)[(size_t)c * sk.Mp];
                                } else {
                                    const float *tt = (const float *)sk.tmt; // [dec][Mp]
                                    const int hs = net.hoff[sk.from];
                                    for (int k = 0; k < net.nodes[sk.from]; ++k)
                                        if (key_bit(key, hs + k)) a -= tt[(size_t)k * sk.Mp] * cr[(size_t)(hs + k) * 4 + c];
                                }
                            }
                            if (c == 3) a += bl - iso;
                            ((float *)ch.eq)[(size_t)(rl0 + rg) * 4 + c] = a;
                        }
                    }
                    bar_builders();
                }
            }
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tslot, (uint32_t)tmem_cols);
}

// src (M x K fp32, row-major) -> three bf16 terms as the shared-memory image
// of 128 x 64 blocks (K-major, 128-byte swizzle), zero padding to Mp x Kp
__global__ void pack_weights_kernel(const float *src, int M, int K, int Mp, int Kp, uint8_t *dst)
{
    const long long n = (long long)Mp * Kp;
    const int kblocks = Kp / 64;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(q / Kp), k = (int)(q % Kp);
        const float v = (m < M && k < K) ? src[(size_t)m * K + k] : 0.f;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h);
        const __nv_bfloat16 md = __float2bfloat16_rn(r1);
        const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(md));
        const int mt = m >> 7, r = m & 127, kb = k >> 6, kk = k & 63;
        uint8_t *blk = dst + (size_t)(mt * kblocks + kb) * kWBlockBytes;
        const uint32_t off = (uint32_t)(r * 128 + ((((kk >> 3) ^ (r & 7)) & 7) << 4) + ((kk & 7) << 1));
        *reinterpret_cast<__nv_bfloat16 *>(blk + off) = h;
        *reinterpret_cast<__nv_bfloat16 *>(blk + 16384 + off) = md;
        *reinterpret_cast<__nv_bfloat16 *>(blk + 32768 + off) = lo;
    }
}

} // namespace

int device_sms()
{
    static int sms[64] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!sms[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        sms[dev] = n > 0 ? n : 148;
    }
    return sms[dev];
}

size_t tc_smem_bytes(const TcNet &tc, int ncols, int W)
{
    if (tc.streamed) { // two operand stages of one K block each (the face-plane sums reuse them)
        const size_t cols = tc.mn ? (size_t)(ncols + 63) / 64 * 64 : (size_t)ncols;
        return 1024 + std::max<size_t>(6 * cols * 64 * 2, (size_t)kSFaceSumBytes) + (size_t)tc.nstage * kWBlockBytes +
               (size_t)(tc.ncols_max / 4) * key_stride(W) * 4 + 16 * (size_t)tc.n1 + 4 * (size_t)tc.k_last + 16;
    }
    const size_t cols = tc.mn ? (size_t)(ncols + 63) / 64 * 64 : (size_t)ncols;
    return 1024 + 3 * cols * tc.kp_max * 2 + (size_t)tc.nstage * kWBlockBytes + (size_t)(tc.ncols_max / 4) * key_stride(W) * 4 +
           16 * (size_t)tc.n1 + 4 * (size_t)tc.k_last + 16 + (size_t)kFaceSumBytes;
}

void launch_compose_tc(const NetDev &net, const TcNet &tc, const RegionsDev &reg, const ChunkDev &ch, double iso,
                       int *d_err, cudaStream_t st)
{
    if (!ch.ctl && ch.count <= 0) return;
    const int sms = device_sms();
    const size_t smem_max = tc_smem_bytes(tc, tc.ncols_max, net.W);
    const int slots = sms; // one resident tile per SM
    if (tc.streamed) {
        cudaFuncSetAttribute(compose_tcs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
        if (ch.ctl) {
            compose_tcs_kernel<<<slots, kSThreads, smem_max, st>>>(net, tc, reg, ch, (float)iso, slots, d_err);
            return;
        }
        const int ncols = tile_cols(ch.count, slots, tc.ncols_max);
        const int R = ncols / 4;
        compose_tcs_kernel<<<(ch.count + R - 1) / R, kSThreads, tc_smem_bytes(tc, ncols, net.W), st>>>(
            net, tc, reg, ch, (float)iso, slots, d_err);
        return;
    }
    cudaFuncSetAttribute(compose_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_max);
    if (ch.ctl) { // wave size known on the device only: every resident tile slot, tiles strided
        compose_tc_kernel<<<slots, kThreads + 32, smem_max, st>>>(net, tc, reg, ch, (float)iso, slots, d_err);
        return;
    }
    const int ncols = tile_cols(ch.count, slots, tc.ncols_max);
    const int R = ncols / 4;
    const int grid = (ch.count + R - 1) / R;
    compose_tc_kernel<<<grid, kThreads + 32, tc_smem_bytes(tc, ncols, net.W), st>>>(net, tc, reg, ch, (float)iso, slots,
                                                                              d_err);
}

void launch_pack_weights(const float *src, int M, int K, int Mp, int Kp, void *dst, cudaStream_t st)
{
    const long long n = (long long)Mp * Kp;
    if (n <= 0) return;
    const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    pack_weights_kernel<<<grid, 256, 0, st>>>(src, M, K, Mp, Kp, (uint8_t *)dst);
}

} // namespace am
