// am_compose_tc.cu -- region affine composition on the 5th-generation tensor
// cores (the mixed-precision form).
//
// Same mathematics as am_compose.cu (the reference's fill_constraints,
// backend/inc/process.h:18-193): for every region, A_{l+1} = W_l diag(s_l) A_l
// (+ b_l, + skips), C = (1 - 2 s) A.  One CTA owns a tile of up to 64 regions
// (4 columns each, N = 4 x regions <= 256) and keeps the masked operand
// X_l = diag(s_l) A_l on chip the whole way through the network: as bf16
// hi/lo splits in 128B-swizzled K-major shared memory, the B operand of
// tcgen05.mma.  The layer weights, pre-split the same way and padded to
// 128-row x 64-column blocks, are the A operand, staged block by block.
// Every operand is split into three bf16 terms, x = hi + mid + lo (24
// significant bits, as fp32); a block issues the six products whose weight is
// at least 2^-16 -- hh, hm, mh, hl, lh, mm.  A two-term split leaves ~2^-17
// of every operand unrepresented, which moved vertices by ~1.5e-5 and changed
// near-degenerate walk decisions.  The tensor core's fp32 accumulation error
// grows with the number of accumulate steps into one accumulator, so the
// dominant hh product and the five small correction products accumulate in
// two separate TMEM accumulators that the epilogue adds once: fp32-level
// constraint rows.  The epilogue reads the accumulators with
// tcgen05.ld (one TMEM lane per output unit), adds bias and skips, writes the
// sign-flipped constraint rows to HBM for the polygon kernel, and writes the
// next layer's masked operand straight back into shared memory.  The face
// plane (output layer, one row) is a 4 x K dot product per region in fp32
// from the rows just written.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"
#include "am_tc.h"
#include "am_umma.cuh"

namespace am {

namespace {

constexpr int kThreads = 128;
constexpr int kWaitIters = 1 << 22;

// x = hi + mid + lo in bf16; the operand buffers are `xbytes` apart
__device__ __forceinline__ void put_split(uint8_t *xs, size_t xbytes, int n, int k, int ncols, float v)
{
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const float r1 = v - __bfloat162float(h);
    const __nv_bfloat16 m = __float2bfloat16_rn(r1);
    const __nv_bfloat16 l = __float2bfloat16_rn(r1 - __bfloat162float(m));
    const uint32_t off = umma::sw128_offset(n, k, ncols);
    *reinterpret_cast<__nv_bfloat16 *>(xs + off) = h;
    *reinterpret_cast<__nv_bfloat16 *>(xs + xbytes + off) = m;
    *reinterpret_cast<__nv_bfloat16 *>(xs + 2 * xbytes + off) = l;
}

// X[n = 4r + c][k] = s_k(r) ? -C[r][src + k][c] : 0 for k < K, 0 up to Kp
__device__ void stage_x_from_rows(uint8_t *xs, size_t xbytes, int ncols, const float *cons, size_t rstride,
                                  const uint32_t *keys, int W, int nreg, int src, int K, int Kp)
{
    const int R = ncols / 4;
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
#pragma unroll
        for (int c = 0; c < 4; ++c) put_split(xs, xbytes, 4 * r + c, k, ncols, x[c]);
    }
}

// one 128-row x 64-column block of a pre-split weight (three terms) into the
// stage buffers (16 KB apart)
__device__ void stage_w_block(uint8_t *ws, const TcMat &m, int mt, int kb)
{
    const size_t plane = (size_t)m.Mp * m.Kp;
    const __nv_bfloat16 *src = m.hi + (size_t)(mt * 128) * m.Kp + (size_t)kb * 64;
    for (int q = threadIdx.x; q < 3 * 128 * 8; q += kThreads) {
        const int t = q / (128 * 8), rq = q % (128 * 8);
        const int row = rq >> 3, ch = rq & 7;
        const uint4 v = *reinterpret_cast<const uint4 *>(src + t * plane + (size_t)row * m.Kp + ch * 8);
        *reinterpret_cast<uint4 *>(ws + t * 16384 + row * 128 + (((ch ^ (row & 7)) & 7) << 4)) = v;
    }
}

struct Pipe {
    uint64_t *bar;
    uint32_t phase;
    int *err;
};

// D[mt] (+)= M . X over all K blocks of the operand in shared memory: six
// products per K step (terms t, u of weight 2^-8(t+u), t + u <= 2)
__device__ void gemm_accumulate(const TcMat &m, int mtiles, uint8_t *ws, uint8_t *xs, size_t xbytes, int ncols,
                                uint32_t tmem, bool first, Pipe &pp)
{
    const uint32_t idesc = umma::idesc_bf16(128, ncols);
    const int kblocks = m.Kp / 64;
    for (int mt = 0; mt < mtiles; ++mt) {
        for (int kb = 0; kb < kblocks; ++kb) {
            stage_w_block(ws, m, mt, kb);
            umma::fence_proxy_async();
            __syncthreads();
            if (threadIdx.x == 0) {
                umma::fence_after();
                const uint32_t a0 = umma::smem_addr(ws);
                const uint32_t b0 = umma::smem_addr(xs) + (uint32_t)(kb * ncols * 128);
                const uint32_t d_main = tmem + (uint32_t)(mt * ncols);            // hh
                const uint32_t d_corr = tmem + (uint32_t)((mtiles + mt) * ncols); // the rest
                const bool fresh = first && kb == 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint32_t o = (uint32_t)(j * 32);
                    umma::mma_bf16(d_main, umma::desc_sw128(a0 + o), umma::desc_sw128(b0 + o), idesc,
                                   (fresh && j == 0) ? 0u : 1u);
                    int q = 0;
#pragma unroll
                    for (int t = 0; t < 3; ++t)
#pragma unroll
                        for (int u = 0; u + t < 3; ++u) {
                            if (t == 0 && u == 0) continue;
                            umma::mma_bf16(d_corr, umma::desc_sw128(a0 + t * 16384u + o),
                                           umma::desc_sw128(b0 + (uint32_t)(u * xbytes) + o), idesc,
                                           (fresh && j == 0 && q == 0) ? 0u : 1u);
                            ++q;
                        }
                }
                umma::commit(umma::smem_addr(pp.bar));
            }
            __syncwarp();
            if (!umma::mbar_wait(pp.bar, pp.phase, kWaitIters)) {
                if (threadIdx.x == 0) atomicOr(pp.err, kErrWalk);
                umma::mbar_wait(pp.bar, pp.phase, kWaitIters);
            }
            pp.phase ^= 1u;
        }
    }
}

__global__ void __launch_bounds__(kThreads, 1) compose_tc_kernel(NetDev net, TcNet tc, RegionsDev reg, ChunkDev ch,
                                                                  float iso, int *err)
{
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t bar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ncols = tc.ncols, R = ncols / 4;
    const long long rl0 = (long long)blockIdx.x * R;
    const int nreg = (int)min((long long)R, (long long)ch.count - rl0);
    if (nreg <= 0) return;
    const size_t rstride = (size_t)net.ALLP * 4;
    float *cons = (float *)ch.cons + (size_t)rl0 * rstride;
    const uint32_t *keys = reg.keys + (size_t)(ch.head + rl0) * net.W;

    uint8_t *base = smem_raw + ((1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u);
    const size_t xbytes = (size_t)ncols * tc.kp_max * 2; // one bf16 term of the operand
    uint8_t *xs = base;                                  // hi, mid, lo: 3 x xbytes
    uint8_t *ws = base + 3 * xbytes;                     // 3 x 16 KB weight block
    uint32_t *skeys = reinterpret_cast<uint32_t *>(ws + 3 * 16384); // the tile's activation bits
    for (int q = tid; q < R * net.W; q += kThreads) skeys[q] = q < nreg * net.W ? keys[q] : 0u;
    keys = skeys;
    __syncthreads(); // every thread reads every region's bits below

    if (tid == 0) umma::mbar_init(&bar, 1);
    if (warp == 0) umma::tmem_alloc(&tslot, (uint32_t)tc.tmem_cols);

    // hidden layer 1 = linear 0 rows (sign-flipped) and the extra constraints
    {
        const float *W0 = (const float *)net.W0;
        const float *b0 = (const float *)net.bias[0];
        const int n1 = net.nodes[1];
        for (int q = tid; q < nreg * n1; q += kThreads) {
            const int rr = q / n1, m = q % n1;
            const float sg = key_bit(keys + (size_t)rr * net.W, m) ? -1.f : 1.f;
            st4<float>(cons + (size_t)rr * rstride + (size_t)m * 4,
                       make_float4(sg * W0[3 * m], sg * W0[3 * m + 1], sg * W0[3 * m + 2], sg * b0[m]));
        }
        const float *we = (const float *)net.w_extra;
        const float *be = (const float *)net.b_extra;
        for (int q = tid; q < nreg * net.E; q += kThreads) {
            const int rr = q / net.E, e = q % net.E;
            st4<float>(cons + (size_t)rr * rstride + (size_t)(net.N + e) * 4,
                       make_float4(we[3 * e], we[3 * e + 1], we[3 * e + 2], be[e]));
        }
        // X_1 = diag(s_1) [W0 | b0]
        const int Kp = (n1 + 63) / 64 * 64;
        for (int q = tid; q < R * Kp; q += kThreads) {
            const int r = q / Kp, k = q % Kp;
            float x[4] = {0.f, 0.f, 0.f, 0.f};
            if (r < nreg && k < n1 && key_bit(keys + (size_t)r * net.W, k)) {
                x[0] = W0[3 * k];
                x[1] = W0[3 * k + 1];
                x[2] = W0[3 * k + 2];
                x[3] = b0[k];
            }
#pragma unroll
            for (int c = 0; c < 4; ++c) put_split(xs, xbytes, 4 * r + c, k, ncols, x[c]);
        }
    }
    umma::fence_proxy_async();
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    Pipe pp{&bar, 0u, err};

    for (int i = 1; i <= net.n_lin - 2; ++i) {
        const int M = net.nodes[i + 1];
        const int mtiles = (M + 127) / 128;
        gemm_accumulate(tc.lin[i], mtiles, ws, xs, xbytes, ncols, tmem, true, pp);
        for (int s = 0; s < net.nskip[i]; ++s) {
            const SkipDev &sk = net.skip[i][s];
            if (sk.kind == 1 && sk.from >= 1) {
                __syncthreads();
                stage_x_from_rows(xs, xbytes, ncols, cons, rstride, keys, net.W, nreg, net.hoff[sk.from],
                                  net.nodes[sk.from], tc.skip[i][s].Kp);
                umma::fence_proxy_async();
                __syncthreads();
                gemm_accumulate(tc.skip[i][s], mtiles, ws, xs, xbytes, ncols, tmem, false, pp);
            }
        }
        umma::fence_after();
        // epilogue: accumulators -> constraint rows (HBM) and the next operand (smem)
        const float *bias = (const float *)net.bias[i];
        const int Kn = (M + 63) / 64 * 64; // next operand's padded K (the face plane reads it too)
        for (int q = tid; q < R * (Kn - M > 0 ? Kn - M : 0); q += kThreads) {
            const int r = q / (Kn - M), k = M + q % (Kn - M);
#pragma unroll
            for (int c = 0; c < 4; ++c) put_split(xs, xbytes, 4 * r + c, k, ncols, 0.f);
        }
        for (int mt = 0; mt < mtiles; ++mt) {
            const int m = mt * 128 + warp * 32 + lane;
            for (int cb = 0; cb < ncols / 16; ++cb) {
                float v[16], vc[16];
                const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
                umma::tmem_ld16(lane_base + (uint32_t)(mt * ncols + cb * 16), v);
                umma::tmem_ld16(lane_base + (uint32_t)((mtiles + mt) * ncols + cb * 16), vc);
#pragma unroll
                for (int z = 0; z < 16; ++z) v[z] += vc[z];
                if (m >= M) continue;
#pragma unroll
                for (int qq = 0; qq < 4; ++qq) {
                    const int r = cb * 4 + qq;
                    float x[4] = {0.f, 0.f, 0.f, 0.f};
                    if (r < nreg) {
                        const uint32_t *key = keys + (size_t)r * net.W;
                        float *cr = cons + (size_t)r * rstride;
                        float o[4] = {v[4 * qq], v[4 * qq + 1], v[4 * qq + 2], v[4 * qq + 3] + bias[m]};
                        for (int s = 0; s < net.nskip[i]; ++s) {
                            const SkipDev &sk = net.skip[i][s];
                            if (sk.kind == 0) {
                                if (sk.from == 0) {
                                    if (m < 3) o[m] += 1.f;
                                } else {
                                    const int row = net.hoff[sk.from] + m;
                                    if (key_bit(key, row)) {
                                        const float4 c = ld4<float>(cr + (size_t)row * 4);
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
                        const int row = net.hoff[i + 1] + m;
                        const bool act = key_bit(key, row);
                        const float sg = act ? -1.f : 1.f;
                        st4<float>(cr + (size_t)row * 4, make_float4(sg * o[0], sg * o[1], sg * o[2], sg * o[3]));
                        if (act) {
                            x[0] = o[0];
                            x[1] = o[1];
                            x[2] = o[2];
                            x[3] = o[3];
                        }
                    }
                    if (Kn > 0) {
#pragma unroll
                        for (int c = 0; c < 4; ++c) put_split(xs, xbytes, 4 * r + c, m, ncols, x[c]);
                    }
                }
            }
        }
        umma::fence_proxy_async();
        umma::fence_before();
        __syncthreads();
        umma::fence_after();
    }

    // face plane: w_eq = W_L . X_L (+ b_L, + connections into the output layer)
    // in fp32, from the operand in shared memory (hi + mid + lo is exact)
    {
        const int i = net.n_lin - 1;
        const int K = net.nodes[i];
        const float *wl = (const float *)net.Wt[i]; // [K][Mp], column 0
        const int Mp = net.Mp[i];
        const float bl = ((const float *)net.bias[i])[0];
        for (int q = tid; q < nreg * 4; q += kThreads) {
            const int r = q >> 2, c = q & 3, n = 4 * r + c;
            float acc = 0.f;
            for (int k = 0; k < K; ++k) {
                const uint32_t off = umma::sw128_offset(n, k, ncols);
                const float x = __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(xs + off)) +
                                __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(xs + xbytes + off)) +
                                __bfloat162float(*reinterpret_cast<const __nv_bfloat16 *>(xs + 2 * xbytes + off));
                acc += __ldg(wl + (size_t)k * Mp) * x;
            }
            const uint32_t *key = keys + (size_t)r * net.W;
            const float *cr = cons + (size_t)r * rstride;
            for (int s = 0; s < net.nskip[i]; ++s) {
                const SkipDev &sk = net.skip[i][s];
                if (sk.kind == 0) {
                    if (sk.from >= 1 && net.nodes[sk.from] == 1 && key_bit(key, net.hoff[sk.from]))
                        acc -= cr[(size_t)net.hoff[sk.from] * 4 + c];
                } else if (sk.from == 0) {
                    if (c < 3) acc += ((const float *)sk.tmt)[(size_t)c * sk.Mp];
                } else {
                    const float *tt = (const float *)sk.tmt; // [dec][Mp]
                    const int hs = net.hoff[sk.from];
                    for (int k = 0; k < net.nodes[sk.from]; ++k)
                        if (key_bit(key, hs + k)) acc -= tt[(size_t)k * sk.Mp] * cr[(size_t)(hs + k) * 4 + c];
                }
            }
            if (c == 3) acc += bl - iso;
            ((float *)ch.eq)[(size_t)(rl0 + r) * 4 + c] = acc;
        }
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, (uint32_t)tc.tmem_cols);
}

__global__ void split_weights_kernel(const float *src, int M, int K, int Mp, int Kp, __nv_bfloat16 *dst)
{
    const long long n = (long long)Mp * Kp;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int m = (int)(q / Kp), k = (int)(q % Kp);
        const float v = (m < M && k < K) ? src[(size_t)m * K + k] : 0.f;
        const __nv_bfloat16 h = __float2bfloat16_rn(v);
        const float r1 = v - __bfloat162float(h);
        const __nv_bfloat16 md = __float2bfloat16_rn(r1);
        dst[q] = h;
        dst[n + q] = md;
        dst[2 * n + q] = __float2bfloat16_rn(r1 - __bfloat162float(md));
    }
}

} // namespace

size_t tc_smem_bytes(const TcNet &tc, int W)
{
    return 1024 + 3 * (size_t)tc.ncols * tc.kp_max * 2 + 3 * 128 * 128 + (size_t)(tc.ncols / 4) * W * 4;
}

void launch_compose_tc(const NetDev &net, const TcNet &tc, const RegionsDev &reg, const ChunkDev &ch, double iso,
                       int *d_err, cudaStream_t st)
{
    if (ch.count <= 0) return;
    const int R = tc.ncols / 4;
    const int grid = (ch.count + R - 1) / R;
    const size_t smem = tc_smem_bytes(tc, net.W);
    cudaFuncSetAttribute(compose_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    compose_tc_kernel<<<grid, kThreads, smem, st>>>(net, tc, reg, ch, (float)iso, d_err);
}

void launch_split_weights(const float *src, int M, int K, int Mp, int Kp, void *dst, cudaStream_t st)
{
    const long long n = (long long)Mp * Kp;
    if (n <= 0) return;
    const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    split_weights_kernel<<<grid, 256, 0, st>>>(src, M, K, Mp, Kp, (__nv_bfloat16 *)dst);
}

} // namespace am
