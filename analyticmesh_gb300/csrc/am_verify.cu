// am_verify.cu -- the per-result error report: max |f(v)| and the largest
// vertex error of a marching result against FP64.
//
// The reference reports marching times only (backend/main.py:368-373).  Here
// a sample of the result's faces is checked against an FP64 evaluation of the
// same network: the sampled regions' constraint rows and face planes are
// composed again in FP64 (the SIMT composition in double, from the engine's
// own copy of the parameters converted exactly to double), and for every
// vertex of such a face
//   * f(v) = w_eq . v + b_eq - iso with the FP64 face plane: the network's
//     value at the output vertex (the region's affine piece is exact at v,
//     which lies in the closure of the region);
//   * v64 = the 3x3 solve, in FP64 from the FP64 rows, of the planes the
//     vertex lies on (the edges entering and leaving it and the face plane);
//     the vertex error is max_c |v_c - v64_c|.
// Vertices of singular systems (|det| below 1e-300) are left out of the
// vertex error and counted.
#include <cuda_runtime.h>

#include <algorithm>

#include "am_device.cuh"
#include "am_internal.h"

namespace am {

namespace {

__global__ void gather_keys_kernel(const uint32_t *keys, int W, const long long *ids, int count, uint32_t *out)
{
    const long long n = (long long)count * W;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q / W), w = (int)(q % W);
        out[q] = keys[(size_t)ids[j] * W + w];
    }
}

__global__ void to_double_kernel(const float *src, long long n, double *dst)
{
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x)
        dst[q] = (double)src[q];
}

// non-negative doubles order like their bit patterns
__device__ __forceinline__ void atomic_max_nonneg(unsigned long long *p, double v)
{
    if (!(v >= 0.0)) v = __longlong_as_double(0x7ff0000000000000ll); // NaN -> +inf: reported, never hidden
    atomicMax(p, (unsigned long long)__double_as_longlong(v));
}

// one thread per (sampled region, vertex slot)
template <typename TS>
__global__ void verify_kernel(RegionsDev reg, const long long *ids, int count, const double *rows, const double *eq,
                              int ALLP, int ALL, unsigned long long *out)
{
    const long long n = (long long)count * kVMax;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(q / kVMax), i = (int)(q % kVMax);
        const long long rid = ids[j];
        const int nv = reg.nv[rid];
        if (nv < 3 || i >= nv || reg.status[rid] != kOk) continue;
        if (i == 0) atomicAdd(out + 4, 1ull); // a face checked
        const TS *vp = (const TS *)reg.verts + ((size_t)rid * kVMax + i) * 3;
        const double v[3] = {(double)vp[0], (double)vp[1], (double)vp[2]};
        const double *e = eq + (size_t)j * 4;
        // the face plane's b already has the level subtracted (b_eq - iso)
        const double f = e[0] * v[0] + e[1] * v[1] + e[2] * v[2] + e[3];
        atomic_max_nonneg(out + 0, fabs(f));
        atomicAdd(out + 2, 1ull);
        const int a = reg.edges[(size_t)rid * kVMax + (i + nv - 1) % nv];
        const int b = reg.edges[(size_t)rid * kVMax + i];
        if (a < 0 || b < 0 || a >= ALL || b >= ALL || a == b) {
            atomicAdd(out + 3, 1ull);
            continue;
        }
        const double *ra = rows + ((size_t)j * ALLP + a) * 4;
        const double *rb = rows + ((size_t)j * ALLP + b) * 4;
        double x[3];
        const double d = solve3<double>(ra, rb, e, x);
        if (!(fabs(d) > 1e-300)) {
            atomicAdd(out + 3, 1ull);
            continue;
        }
        const double err = fmax(fabs(v[0] - x[0]), fmax(fabs(v[1] - x[1]), fabs(v[2] - x[2])));
        atomic_max_nonneg(out + 1, err);
    }
}

int grid_for(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 8ll * device_sms())); }

} // namespace

void launch_gather_keys(const uint32_t *keys, int W, const long long *ids, int count, uint32_t *out, cudaStream_t st)
{
    if (count <= 0) return;
    gather_keys_kernel<<<grid_for((long long)count * W), 256, 0, st>>>(keys, W, ids, count, out);
}

void launch_to_double(const void *src, long long n, void *dst, cudaStream_t st)
{
    if (n <= 0) return;
    to_double_kernel<<<grid_for(n), 256, 0, st>>>((const float *)src, n, (double *)dst);
}

void launch_verify(int ts_bytes, const RegionsDev &reg, const long long *ids, int count, const double *rows,
                   const double *eq, int ALLP, int ALL, unsigned long long *out, cudaStream_t st)
{
    if (count <= 0) return;
    const long long n = (long long)count * kVMax;
    if (ts_bytes == 8)
        verify_kernel<double><<<grid_for(n), 256, 0, st>>>(reg, ids, count, rows, eq, ALLP, ALL, out);
    else
        verify_kernel<float><<<grid_for(n), 256, 0, st>>>(reg, ids, count, rows, eq, ALLP, ALL, out);
}

} // namespace am
