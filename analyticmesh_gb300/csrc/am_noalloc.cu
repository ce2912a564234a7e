// am_noalloc.cu -- region composition without any device allocation.
//
// For callers that cannot call cudaMalloc: code running inside a host
// framework that owns every byte of device memory through its own pool, or
// under a fixed memory budget where a hidden allocation would fail or
// fragment it, or in a callback where allocating (an implicitly synchronising
// call) is not allowed.  They pass their own device inputs and outputs; the
// scratch this composition needs -- the transposed weights the SIMT kernel
// reads and the packed activation keys -- lives in one file-scope device
// array of fixed size instead of engine buffers.
//
// The array is part of this library's device image: every GPU that loads the
// library holds its 8 MiB until the process exits.  Its device address is
// looked up once per device, on the first call made with that device
// current; that first call should therefore happen before any stream capture.
// All calls share the array and it keeps the last call's contents; nothing in
// it has to start at zero (each call writes every scratch byte it reads).
// Calls whose work overlaps on the GPU (other streams, or the same stream
// from other threads without ordering) race on the array.  The looked-up
// address belongs to the device's current context: after cudaDeviceReset
// (or anything else that destroys the primary context) it is stale, and the
// entry point must not be called again in that process.
//
// Errors: a CUDA error already pending on the calling thread is reported as
// AM_ERR_CUDA without launching anything and is left pending for its owner;
// otherwise the status covers this call's launches only.  A non-null stream
// must belong to the current device (AM_ERR_INVALID_ARGUMENT otherwise).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <mutex>

#include "../../include/analyticmesh_gb300.h"
#include "am_internal.h"

namespace am {
namespace {

constexpr size_t kScratchBytes = size_t(8) << 20;
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
void *g_scratch_addr[kMaxDevices] = {};
std::mutex g_scratch_mu;

size_t align256(size_t n) { return (n + 255) / 256 * 256; }

} // namespace
} // namespace am

extern "C" int am_compose_rows_noalloc(const int32_t *nodesnum, int num_nodes, const float *const *weights,
                                       const float *const *biases, const uint8_t *states, int count, double iso,
                                       float *rows, float *eq, void *stream)
{
    using namespace am;
    if (!nodesnum || num_nodes < 3 || num_nodes - 1 > kMaxLayers || nodesnum[0] != 3 || nodesnum[num_nodes - 1] != 1)
        return AM_ERR_INVALID_ARGUMENT;
    if (!weights || !biases || !states || !rows || !eq || count < 1) return AM_ERR_INVALID_ARGUMENT;
    if (((uintptr_t)rows & 15u) || ((uintptr_t)eq & 15u)) return AM_ERR_INVALID_ARGUMENT;
    const int n_lin = num_nodes - 1;
    int N = 0;
    for (int i = 1; i < n_lin; ++i) {
        if (nodesnum[i] <= 0) return AM_ERR_INVALID_ARGUMENT;
        N += nodesnum[i];
    }
    for (int i = 0; i < n_lin; ++i)
        if (!weights[i] || !biases[i]) return AM_ERR_INVALID_ARGUMENT;
    const int W = (N + 31) / 32;

    // scratch layout: transposed weights of linears 1.., then keys, then key hashes
    size_t off[kMaxLayers] = {};
    size_t used = 0;
    for (int i = 1; i < n_lin; ++i) {
        const int Mp = (nodesnum[i + 1] + 3) / 4 * 4;
        off[i] = used;
        used += align256(sizeof(float) * (size_t)nodesnum[i] * Mp);
    }
    const size_t keys_off = used;
    used += align256(sizeof(uint32_t) * (size_t)count * W);
    const size_t hash_off = used;
    used += align256(sizeof(uint64_t) * (size_t)count);
    if (used > kScratchBytes) return AM_ERR_CAPACITY; // network + states larger than the 8 MiB scratch

    // an error left pending by earlier work is not ours to report or to clear
    if (cudaPeekAtLastError() != cudaSuccess) return AM_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return AM_ERR_CUDA;
    if (stream) {
        int sdev = -1;
        if (cudaStreamGetDevice((cudaStream_t)stream, &sdev) != cudaSuccess) return AM_ERR_INVALID_ARGUMENT;
        if (sdev != dev) return AM_ERR_INVALID_ARGUMENT;
    }
    unsigned char *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[dev]) {
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_scratch) != cudaSuccess || !p) return AM_ERR_CUDA;
            g_scratch_addr[dev] = p;
        }
        scratch = (unsigned char *)g_scratch_addr[dev];
    }
    cudaStream_t st = (cudaStream_t)stream;

    NetDev net;
    memset(&net, 0, sizeof(net));
    net.n_lin = n_lin;
    net.N = N;
    net.E = 0;
    net.ALL = N;
    net.ALLP = N; // rows are packed: count x N x 4
    net.W = W;
    for (int i = 0; i <= n_lin; ++i) net.nodes[i] = nodesnum[i];
    net.hoff[1] = 0;
    for (int h = 1; h < n_lin; ++h) net.hoff[h + 1] = net.hoff[h] + nodesnum[h];
    net.W0 = weights[0];
    for (int i = 0; i < n_lin; ++i) net.bias[i] = biases[i];
    for (int i = 1; i < n_lin; ++i) {
        const int M = nodesnum[i + 1], K = nodesnum[i], Mp = (M + 3) / 4 * 4;
        launch_prepare_weights(kFloat32, weights[i], M, K, Mp, scratch + off[i], st);
        net.Wt[i] = scratch + off[i];
        net.Mp[i] = Mp;
    }
    uint32_t *keys = (uint32_t *)(scratch + keys_off);
    uint64_t *hash = (uint64_t *)(scratch + hash_off);
    launch_seed_pack(states, count, N, W, keys, hash, st);

    RegionsDev reg;
    memset(&reg, 0, sizeof(reg));
    reg.keys = keys;
    reg.hash = hash;
    reg.cap = count;
    ChunkDev ch;
    ch.head = 0;
    ch.count = count;
    ch.cons = rows;
    ch.eq = eq;
    ch.rec = nullptr;
    launch_compose(kFloat32, net, reg, ch, iso, st);
    // nothing was pending at entry: an error now comes from these launches
    return cudaGetLastError() == cudaSuccess ? AM_OK : AM_ERR_CUDA;
}
