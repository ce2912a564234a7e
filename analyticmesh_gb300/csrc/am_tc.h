// am_tc.h -- network layout for the tensor-core composition (mixed form).
#pragma once

#include <cstddef>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "am_internal.h"

namespace am {

// A weight pre-split into three bf16 terms (w = hi + mid + lo, 24 bits),
// zero-padded to Mp (multiple of 128) rows x Kp (multiple of 64) columns,
// row-major; the three planes are contiguous starting at `hi`.
struct TcMat {
    const __nv_bfloat16 *hi;
    int Mp, Kp;
};

struct TcNet {
    TcMat lin[kMaxLayers];              // linear i, 1 <= i <= n_lin - 2 (hidden outputs)
    TcMat skip[kMaxLayers][kMaxSkips];  // transforms from hidden layers into linear i
    int ncols;                          // UMMA N = 4 x regions per CTA (multiple of 16, <= 256)
    int kp_max;                         // largest padded K of any operand
    int tmem_cols;                      // TMEM columns per CTA (power of two)
};

size_t tc_smem_bytes(const TcNet &tc, int W);
void launch_compose_tc(const NetDev &net, const TcNet &tc, const RegionsDev &reg, const ChunkDev &ch, double iso,
                       int *d_err, cudaStream_t st);
void launch_split_weights(const float *src, int M, int K, int Mp, int Kp, void *dst, cudaStream_t st);

} // namespace am
