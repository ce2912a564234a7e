// am_tc.h -- network layout for the tensor-core composition (mixed form).
#pragma once

#include <cstddef>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "am_internal.h"

namespace am {

// A weight pre-split into three bf16 terms (w = hi + mid + lo, 24 bits),
// zero-padded to Mp (multiple of 128) rows x Kp (multiple of 64) columns and
// stored as the shared-memory image of its 128 x 64 blocks: block (mt, kb)
// at (mt * Kp / 64 + kb) * kWBlockBytes holds the three terms 16 KB apart,
// each K-major with the 128-byte swizzle, so one bulk copy stages it.
constexpr int kWBlockBytes = 3 * 128 * 128;

struct TcMat {
    const uint8_t *blocks;
    int Mp, Kp;
};

struct TcNet {
    TcMat lin[kMaxLayers];              // linear i, 1 <= i <= n_lin - 2 (hidden outputs)
    TcMat skip[kMaxLayers][kMaxSkips];  // transforms from hidden layers into linear i
    int ncols_max;                      // widest UMMA N = 4 x regions per CTA (multiple of 16, <= 256)
    int kp_max;                         // largest padded K of any operand
    int mtiles_max;                     // largest number of 128-row tiles of any layer
    int nstage;                         // weight blocks in flight (1 or 2; up to 3 with the streamed operand)
    int mn;                             // operand layout: 1 MN-major (64-column atoms), 0 K-major
    int n1, k_last;                     // widths of hidden layer 1 and of the last hidden layer
    int streamed;                       // operand rebuilt per 64-wide K block from the rows (wide layers)
    int mgroups;                        // streamed: a layer's M tiles in this many passes, each with its own
                                        // accumulators (TMEM holds 2 x ceil(mtiles / mgroups) x ncols columns)
};

size_t tc_smem_bytes(const TcNet &tc, int ncols, int W);
void launch_compose_tc(const NetDev &net, const TcNet &tc, const RegionsDev &reg, const ChunkDev &ch, double iso,
                       int *d_err, cudaStream_t st);
void launch_pack_weights(const float *src, int M, int K, int Mp, int Kp, void *dst, cudaStream_t st);

} // namespace am
