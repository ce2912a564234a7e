// am_compose.cu -- region affine composition (SIMT form, fp32 / fp64).
//
// For every region of a chunk, compose the affine map of every hidden unit
// under the region's activation state and write the sign-flipped constraint
// rows C_k = (1 - 2 s_k) [w_k | b_k] plus the face plane (w_eq, b_eq - iso).
// Same mathematics as the reference's fill_constraints + offset_b_equ
// (backend/inc/process.h:18-203), organised GB300-first: one CTA composes 16
// regions through every layer, the layer product W_l . diag(s_l) A_l runs as
// a 64-row x 64-column register-tiled product with the masked operand
// diag(s_l) A_l = -s_l * C_l staged in shared memory, and skip connections
// accumulate into the same tile.  Connections into the output layer are
// composed too (the reference's loop stops before them, process.h:42).
#include <algorithm>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"

namespace am {

namespace {

constexpr int kR = 16;        // regions per CTA
constexpr int kThreads = 256; // 16 regions x 16 row groups of 4 rows
constexpr int kKC = 32;       // k rows staged per pass
constexpr int kRowsPerPass = 64;

template <typename T>
struct Acc {
    T v[4][4];
};

// acc[j][c] += sum_k Wt[k][m0 + j] * X[k][c] for the thread's region, where
// X = diag(s) rows [src, src+K) of the region's constraint block, negated
// (C = -A for active units, so s * A = -s * C).
template <typename T>
__device__ __forceinline__ void accumulate(vec4_t<T> (*X)[kR], const T *cons, size_t rstride, const uint32_t *keys, int W,
                                           int nreg, int src, int K, const T *Wt, int Mp, int m0, Acc<T> &acc)
{
    const int tid = threadIdx.x;
    const int r = tid & (kR - 1);
    const bool has_w = m0 < Mp;
    for (int k0 = 0; k0 < K; k0 += kKC) {
        const int kc = min(kKC, K - k0);
        __syncthreads();
        for (int q = tid; q < kKC * kR; q += kThreads) {
            const int rr = q / kKC, kk = q % kKC;
            vec4_t<T> x;
            x.x = x.y = x.z = x.w = T(0);
            if (kk < kc && rr < nreg) {
                const int row = src + k0 + kk;
                if (key_bit(keys + (size_t)rr * W, row)) {
                    const vec4_t<T> c = ld4<T>(cons + (size_t)rr * rstride + (size_t)row * 4);
                    x.x = -c.x;
                    x.y = -c.y;
                    x.z = -c.z;
                    x.w = -c.w;
                }
            }
            X[kk][rr] = x;
        }
        __syncthreads();
        if (has_w) {
            const T *wp = Wt + (size_t)k0 * Mp + m0;
#pragma unroll 4
            for (int kk = 0; kk < kc; ++kk) {
                const vec4_t<T> x = X[kk][r];
                const vec4_t<T> w = ld4<T>(wp + (size_t)kk * Mp);
                const T wj[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    acc.v[j][0] += wj[j] * x.x;
                    acc.v[j][1] += wj[j] * x.y;
                    acc.v[j][2] += wj[j] * x.z;
                    acc.v[j][3] += wj[j] * x.w;
                }
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) compose_kernel(NetDev net, RegionsDev reg, ChunkDev ch, T iso)
{
    __shared__ vec4_t<T> X[kKC][kR];
    const int tid = threadIdx.x;
    const int r = tid & (kR - 1);
    const int g = tid >> 4;
    long long head;
    int count;
    chunk_range(ch, head, count);
    const size_t rstride = (size_t)net.ALLP * 4;
    // tiles of kR regions, strided over the grid (the graph-driven loop
    // launches a fixed grid; the host-driven one a tile per CTA)
    for (long long rl0 = (long long)blockIdx.x * kR; rl0 < count; rl0 += (long long)gridDim.x * kR) {
        const int nreg = (int)min((long long)kR, (long long)count - rl0);
        T *cons = (T *)ch.cons + (size_t)rl0 * rstride;
        const uint32_t *keys = reg.keys + (size_t)(head + rl0) * net.W;

        // hidden layer 1 = linear 0 rows, sign-flipped; extra constraints as given
        {
            const T *W0 = (const T *)net.W0;
            const T *b0 = (const T *)net.bias[0];
            const int n1 = net.nodes[1];
            for (int q = tid; q < nreg * n1; q += kThreads) {
                const int rr = q / n1, m = q % n1;
                const T sg = key_bit(keys + (size_t)rr * net.W, m) ? T(-1) : T(1);
                vec4_t<T> c;
                c.x = sg * W0[3 * m + 0];
                c.y = sg * W0[3 * m + 1];
                c.z = sg * W0[3 * m + 2];
                c.w = sg * b0[m];
                st4<T>(cons + (size_t)rr * rstride + (size_t)m * 4, c);
            }
            const T *we = (const T *)net.w_extra;
            const T *be = (const T *)net.b_extra;
            for (int q = tid; q < nreg * net.E; q += kThreads) {
                const int rr = q / net.E, e = q % net.E;
                vec4_t<T> c;
                c.x = we[3 * e + 0];
                c.y = we[3 * e + 1];
                c.z = we[3 * e + 2];
                c.w = be[e];
                st4<T>(cons + (size_t)rr * rstride + (size_t)(net.N + e) * 4, c);
            }
        }

        for (int i = 1; i < net.n_lin; ++i) {
            const int M = net.nodes[i + 1];
            const int K = net.nodes[i];
            const bool last = (i == net.n_lin - 1);
            const T *bias = (const T *)net.bias[i];
            for (int mb = 0; mb < M; mb += kRowsPerPass) {
                const int m0 = mb + 4 * g;
                Acc<T> acc;
    #pragma unroll
                for (int j = 0; j < 4; ++j)
    #pragma unroll
                    for (int c = 0; c < 4; ++c) acc.v[j][c] = T(0);
                accumulate<T>(X, cons, rstride, keys, net.W, nreg, net.hoff[i], K, (const T *)net.Wt[i], net.Mp[i], m0, acc);
                for (int s = 0; s < net.nskip[i]; ++s) {
                    const SkipDev &sk = net.skip[i][s];
                    if (sk.kind == 1 && sk.from >= 1)
                        accumulate<T>(X, cons, rstride, keys, net.W, nreg, net.hoff[sk.from], net.nodes[sk.from],
                                      (const T *)sk.tmt, sk.Mp, m0, acc);
                }
                if (r < nreg) {
                    const uint32_t *key = keys + (size_t)r * net.W;
                    T *cr = cons + (size_t)r * rstride;
    #pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        const int m = m0 + j;
                        if (m >= M) continue;
                        T v[4] = {acc.v[j][0], acc.v[j][1], acc.v[j][2], acc.v[j][3] + bias[m]};
                        for (int s = 0; s < net.nskip[i]; ++s) {
                            const SkipDev &sk = net.skip[i][s];
                            if (sk.kind == 0) {
                                if (sk.from == 0) {
                                    if (m < 3) v[m] += T(1);
                                } else {
                                    const int row = net.hoff[sk.from] + m;
                                    if (key_bit(key, row)) {
                                        const vec4_t<T> c = ld4<T>(cr + (size_t)row * 4);
                                        v[0] -= c.x;
                                        v[1] -= c.y;
                                        v[2] -= c.z;
                                        v[3] -= c.w;
                                    }
                                }
                            } else if (sk.from == 0) {
                                const T *tt = (const T *)sk.tmt; // [3][Mp]
                                v[0] += tt[m];
                                v[1] += tt[(size_t)sk.Mp + m];
                                v[2] += tt[2 * (size_t)sk.Mp + m];
                            }
                        }
                        vec4_t<T> o;
                        if (!last) {
                            const int row = net.hoff[i + 1] + m;
                            const T sg = key_bit(key, row) ? T(-1) : T(1);
                            o.x = sg * v[0];
                            o.y = sg * v[1];
                            o.z = sg * v[2];
                            o.w = sg * v[3];
                            st4<T>(cr + (size_t)row * 4, o);
                        } else {
                            o.x = v[0];
                            o.y = v[1];
                            o.z = v[2];
                            o.w = v[3] - iso;
                            st4<T>((T *)ch.eq + (size_t)(rl0 + r) * 4, o);
                        }
                    }
                }
            }
            __syncthreads(); // layer i+1 rows written by this CTA become the next operand
        }
    }
}

template <typename T>
__global__ void prepare_weights_kernel(const T *src, int M, int K, int Mp, T *dst)
{
    // dst[k][m] = src[m][k], zero padding for m >= M
    const long long n = (long long)K * Mp;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(q / Mp), m = (int)(q % Mp);
        dst[q] = m < M ? src[(size_t)m * K + k] : T(0);
    }
}

// every value of the listed buffers finite; kErrNonFinite otherwise
template <typename T>
__global__ void check_finite_kernel(FiniteList list, int *err)
{
    const int b = blockIdx.y;
    const T *p = (const T *)list.p[b];
    bool bad = false;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < list.n[b]; q += (long long)gridDim.x * blockDim.x)
        bad |= !isfinite(p[q]);
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(err, kErrNonFinite);
}

} // namespace

void launch_check_finite(int prec, const FiniteList &list, int *d_err, cudaStream_t st)
{
    if (list.count <= 0) return;
    long long most = 1;
    for (int b = 0; b < list.count; ++b) most = std::max(most, list.n[b]);
    const dim3 grid((unsigned)std::min<long long>((most + 255) / 256, 64), (unsigned)list.count);
    if (prec == kFloat64)
        check_finite_kernel<double><<<grid, 256, 0, st>>>(list, d_err);
    else
        check_finite_kernel<float><<<grid, 256, 0, st>>>(list, d_err);
}

void launch_compose(int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, double iso, cudaStream_t st)
{
    if (!ch.ctl && ch.count <= 0) return;
    const int grid = ch.ctl ? device_sms() * 4 : (ch.count + kR - 1) / kR;
    if (prec == kFloat64)
        compose_kernel<double><<<grid, kThreads, 0, st>>>(net, reg, ch, iso);
    else
        compose_kernel<float><<<grid, kThreads, 0, st>>>(net, reg, ch, (float)iso);
}

void launch_prepare_weights(int prec, const void *src, int M, int K, int Mp, void *dst, cudaStream_t st)
{
    const long long n = (long long)K * Mp;
    if (n <= 0) return;
    const int grid = (int)std::min<long long>((n + 255) / 256, 4096);
    if (prec == kFloat64)
        prepare_weights_kernel<double><<<grid, 256, 0, st>>>((const double *)src, M, K, Mp, (double *)dst);
    else
        prepare_weights_kernel<float><<<grid, 256, 0, st>>>((const float *)src, M, K, Mp, (float *)dst);
}

} // namespace am
