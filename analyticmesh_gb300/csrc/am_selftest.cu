// am_selftest.cu -- self-test of the tensor-core tile the composition uses:
// one CTA computes D (128 x N, fp32) = A (128 x K, bf16) . B (N x K, bf16)^T
// with tcgen05.mma from K-major 128-byte-swizzled shared memory into TMEM.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/analyticmesh_gb300.h"
#include "am_umma.cuh"

namespace am {
namespace {

__global__ void __launch_bounds__(128) umma_selftest_kernel(const __nv_bfloat16 *A, const __nv_bfloat16 *B, float *D,
                                                             int N, int K, uint32_t ncols, int bmn, int *status)
{
    extern __shared__ uint8_t smem_raw[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tslot;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    uint8_t *base = smem_raw + ((1024u - (umma::smem_addr(smem_raw) & 1023u)) & 1023u);
    uint8_t *sA = base;
    uint8_t *sB = sA + 128 * K * 2;
    for (int q = tid; q < 128 * K; q += 128) {
        const int r = q / K, k = q % K;
        *reinterpret_cast<__nv_bfloat16 *>(sA + umma::sw128_offset(r, k, 128)) = A[q];
    }
    const int natoms = (N + 63) / 64;
    for (int q = tid; q < N * K; q += 128) {
        const int r = q / K, k = q % K;
        const uint32_t off = bmn ? umma::mn_sw128_offset(r, k, natoms) : umma::sw128_offset(r, k, N);
        *reinterpret_cast<__nv_bfloat16 *>(sB + off) = B[q];
    }
    umma::fence_proxy_async();
    if (tid == 0) umma::mbar_init(&mbar, 1);
    if (warp == 0) umma::tmem_alloc(&tslot, ncols);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tslot;
    if (tid == 0) {
        const uint32_t idesc = bmn ? umma::idesc_bf16_bmn(128, N) : umma::idesc_bf16(128, N);
        for (int j = 0; j < K / 16; ++j) {
            const uint32_t off = (uint32_t)((j & 3) * 32);
            const uint64_t ad = umma::desc_sw128(umma::smem_addr(sA) + (j >> 2) * 128 * 128 + off);
            // MN-major: one K step of 16 is two 8-row groups
            const uint64_t bd = bmn ? umma::desc_sw128_mn(umma::smem_addr(sB) + (uint32_t)(2 * j * natoms * 1024), 1024u,
                                                          (uint32_t)(natoms * 1024))
                                    : umma::desc_sw128(umma::smem_addr(sB) + (j >> 2) * N * 128 + off);
            umma::mma_bf16(tmem, ad, bd, idesc, j > 0 ? 1u : 0u);
        }
        umma::commit(umma::smem_addr(&mbar));
    }
    __syncwarp();
    if (!umma::mbar_wait(&mbar, 0, 1 << 20)) {
        atomicOr(status, 1);
        umma::mbar_wait(&mbar, 0, 1 << 20); // give the tensor core a second bound before freeing TMEM
    }
    umma::fence_after();
    const int row = warp * 32 + lane;
    for (int c0 = 0; c0 < N; c0 += 16) {
        float v[16];
        umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
#pragma unroll
        for (int i = 0; i < 16; ++i) D[(size_t)row * N + c0 + i] = v[i];
    }
    umma::fence_before();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}

} // namespace
} // namespace am

namespace {
int selftest(const void *A, const void *B, void *D, int N, int K, int bmn)
{
    if (N < 16 || N > 256 || N % 16 || K < 64 || K % 64) return AM_ERR_INVALID_ARGUMENT;
    uint32_t ncols = 32;
    while (ncols < (uint32_t)N) ncols <<= 1;
    int *status = nullptr;
    if (cudaMalloc(&status, sizeof(int)) != cudaSuccess) return AM_ERR_OUT_OF_MEMORY;
    cudaMemset(status, 0, sizeof(int));
    // B region: N x K (K-major) or 64-wide atoms (MN-major), doubled so that
    // every descriptor reading of it stays inside the allocation
    const size_t bbytes = (size_t)(bmn ? (N + 63) / 64 * 64 : N) * K * 2;
    const size_t smem = 1024 + (size_t)128 * K * 2 + 2 * bbytes;
    cudaFuncSetAttribute(am::umma_selftest_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    am::umma_selftest_kernel<<<1, 128, smem>>>((const __nv_bfloat16 *)A, (const __nv_bfloat16 *)B, (float *)D, N, K, ncols,
                                               bmn, status);
    cudaError_t e = cudaDeviceSynchronize();
    int h = 0;
    cudaMemcpy(&h, status, sizeof(int), cudaMemcpyDeviceToHost);
    cudaFree(status);
    if (e != cudaSuccess) return AM_ERR_CUDA;
    return h ? AM_ERR_CUDA : AM_OK;
}
} // namespace

extern "C" int am_selftest_umma(const void *A, const void *B, void *D, int N, int K)
{
    return selftest(A, B, D, N, K, 0);
}

extern "C" int am_selftest_umma_bmn(const void *A, const void *B, void *D, int N, int K)
{
    return selftest(A, B, D, N, K, 1);
}
