// am_engine.cpp -- host driver of the GB300 Analytic Marching engine and the
// C ABI declared in include/analyticmesh_gb300.h.
//
// The marching loop processes the append-only region store FIFO in chunks:
// compose every region of the chunk, build its face polygon and insert its
// neighbours, append the new regions at the tail.  One stream, no host work
// inside a chunk; the host reads the new tail once per chunk.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstdio>
#include <climits>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/analyticmesh_gb300.h"
#include "am_internal.h"
#include "am_mesh.h"
#include "am_tc.h"

using namespace am;

namespace {

// While a batch runs, device frees wait until its end: cudaFree synchronises
// the whole device and would stall every other network's stream.
thread_local std::vector<void *> *t_deferred_frees = nullptr;

void release_device(void *p)
{
    if (!p) return;
    if (t_deferred_frees) t_deferred_frees->push_back(p);
    else cudaFree(p);
}

struct DeferFrees {
    std::vector<void *> list;
    DeferFrees() { t_deferred_frees = &list; }
    ~DeferFrees()
    {
        t_deferred_frees = nullptr;
        if (!list.empty()) cudaDeviceSynchronize();
        for (void *p : list) cudaFree(p);
    }
};

// A device allocation.  Inside a batch, allocations that take a stream come
// from the stream-ordered pool (cudaMallocAsync) and go back to it in stream
// order (cudaFreeAsync), so that a network's growing stores neither stall
// the other networks' streams (as cudaFree would) nor wait for the batch's
// end to be freed.
struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaStream_t pst = nullptr; // pooled: the stream the allocation is ordered on
    bool pooled = false;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf() { reset(); }
    static void release(void *q, bool pool, cudaStream_t qst)
    {
        if (!q) return;
        if (pool) cudaFreeAsync(q, qst);
        else release_device(q);
    }
    void reset()
    {
        release(p, pooled, pst);
        p = nullptr;
        bytes = 0;
        pooled = false;
        pst = nullptr;
    }
    static cudaError_t get(void **q, size_t n, cudaStream_t st, bool &pool)
    {
        pool = st && t_deferred_frees;
        return pool ? cudaMallocAsync(q, n, st) : cudaMalloc(q, n);
    }
    cudaError_t alloc(size_t n, cudaStream_t st = nullptr)
    {
        reset();
        if (n == 0) n = 16;
        bool pool = false;
        cudaError_t e = get(&p, n, st, pool);
        if (e == cudaSuccess) {
            bytes = n;
            pooled = pool;
            pst = pool ? st : nullptr;
        } else {
            p = nullptr;
        }
        return e;
    }
    // at least n bytes, reusing the allocation when it is large enough
    // (contents not kept)
    cudaError_t reserve(size_t n, cudaStream_t st = nullptr)
    {
        if (p && n <= bytes) return cudaSuccess;
        return alloc(n, st);
    }
    // grow keeping the first `keep` bytes
    cudaError_t grow(size_t n, size_t keep, cudaStream_t st)
    {
        if (n <= bytes) return cudaSuccess;
        void *q = nullptr;
        bool pool = false;
        cudaError_t e = get(&q, n, st, pool);
        if (e != cudaSuccess) return e;
        if (p && keep) {
            e = cudaMemcpyAsync(q, p, std::min(keep, bytes), cudaMemcpyDeviceToDevice, st);
            if (e != cudaSuccess) {
                release(q, pool, st);
                return e;
            }
            cudaStreamSynchronize(st);
        }
        release(p, pooled, pst);
        p = q;
        bytes = n;
        pooled = pool;
        pst = pool ? st : nullptr;
        return cudaSuccess;
    }
    template <class T>
    T *as() const
    {
        return (T *)p;
    }
};

struct Failure {
    int code;
    std::string msg;
};

#define AM_CUDA(x)                                                                                \
    do {                                                                                          \
        cudaError_t e_ = (x);                                                                     \
        if (e_ != cudaSuccess) {                                                                  \
            throw Failure{e_ == cudaErrorMemoryAllocation ? AM_ERR_OUT_OF_MEMORY : AM_ERR_CUDA,   \
                          std::string(#x) + ": " + cudaGetErrorString(e_)};                       \
        }                                                                                         \
    } while (0)

#define AM_CHECK(cond, msg)                                                     \
    do {                                                                        \
        if (!(cond)) throw Failure{AM_ERR_INVALID_ARGUMENT, std::string(msg)}; \
    } while (0)

bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// copy n bytes from a host or device pointer to a device buffer
void upload(DevBuf &dst, const void *src, size_t n, cudaStream_t st)
{
    AM_CUDA(dst.reserve(n));
    if (n) AM_CUDA(cudaMemcpyAsync(dst.p, src, n, is_device_ptr(src) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
}

void to_host(void *dst, const void *src, size_t n, cudaStream_t st)
{
    if (!n) return;
    AM_CUDA(cudaMemcpyAsync(dst, src, n, is_device_ptr(src) ? cudaMemcpyDeviceToHost : cudaMemcpyHostToHost, st));
}

} // namespace

struct am_engine {
    int prec = kFloat32;
    std::vector<int> nodes;
    std::vector<int32_t> arc;
    int arc_cols = 1;
    int n_lin = 0, N = 0, E = 0, ALL = 0, ALLP = 0, W = 0;
    size_t tc = 4, ts = 4; // constraint / solve element sizes
    cudaStream_t own = nullptr, st = nullptr;
    std::string last_error;
    int64_t chunk_opt = 0;
    bool phase_timing = false;
    int weld_mode = 0;

    // network
    DevBuf wt[kMaxLayers], bias[kMaxLayers], w0, tmt[64], wext, bext, scratch;
    NetDev net{};
    int ntm = 0;                // transforms in tmt
    long long tm_count[64] = {}; // elements of each
    // error report: FP64 copies of the parameters (FP32 engines), sample buffers
    DevBuf wt64[kMaxLayers], bias64[kMaxLayers], w0_64, tmt64[64], wext64, bext64;
    DevBuf v_ids, v_keys, v_rows, v_eq, v_out;
    // tensor-core composition (mixed form): bf16 hi/lo weights
    DevBuf tc_lin[kMaxLayers], tc_skip[kMaxLayers][kMaxSkips];
    TcNet tcnet{};
    // regions
    DevBuf keys, hash, mid, start, nv, status, verts, edges;
    long long cap = 0;
    DevBuf table;
    unsigned long long hcap = 0;
    // chunk
    DevBuf cons, eq, rec, blocksum;
    int chunk_cap = 0;
    // seeds
    DevBuf s_states, s_keys, s_hash, s_pts, s_rec;
    // counters
    // wave control block (region tail, error bits, the graph-driven loop's
    // queue state), read back with one copy into pinned host memory
    DevBuf d_tail; // the WaveCtl; tail at offset 0
    struct {
        void *p = nullptr;
        template <typename T> T *as() const { return (T *)p; }
    } d_err;
    WaveCtl *h_ctl = nullptr;
    bool use_graph = true;
    // the run in progress: am_analytic_marching, or one network of am_run_batch
    struct Run {
        int prec = 0;
        double iso = 0;
        Tolerances tol{};
        int chunk = 0;
        long long head = 0, tail = 0, launches = 0;
        int chunks = 0;
        double t_comp = 0, t_poly = 0, t_front = 0;
        bool flip = false;
        bool lean = false; // batch member: the wave buffers grow with the queue
    } run;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, pa = nullptr, pb = nullptr;
    bool lean = false; // batch member: region store and table start small and grow on demand
    long long max_regions = 0; // AM_OPT_MAX_REGIONS (0: no limit)
    int compose_tile = 0;      // AM_OPT_COMPOSE_TILE: 0 automatic, 1 resident operand, 2 streamed operand
    int face_warps = 0;        // AM_OPT_FACE_WARPS: warps per face polygon, 0 automatic
    long long table_slots = 0; // AM_OPT_TABLE_SLOTS: fixed region hash table size, 0 automatic
    int inject_err = 0;        // AM_OPT_INJECT_ERROR: error bits set in the control block after the seeds
    int prune = 0;             // AM_OPT_PRUNE_ROWS: the walk scans only the rows that can bound the face
    bool limit_hit = false;    // the last run stopped at the region limit
    bool over_limit(long long tail)
    {
        if (max_regions > 0 && tail > max_regions) limit_hit = true;
        return limit_hit;
    }
    void ensure_events()
    {
        for (cudaEvent_t *ev : {&ev0, &ev1, &pa, &pb})
            if (!*ev) AM_CUDA(cudaEventCreate(ev));
    }
    // the instantiated wave-loop graph and the launch parameters it captured
    cudaGraph_t wgraph = nullptr;
    cudaGraphExec_t wexec = nullptr;
    std::vector<unsigned char> wsig;
    // results
    bool has_am = false, has_mesh = false;
    long long num_regions = 0;
    am_stats stats{};
    int flip = 0;
    double iso = 0.0;
    // mesh
    DevBuf w_table, w_rep, w_flag, w_vidx, w_bsum, w_fflag, w_fsize, w_fid, w_foff, w_verts, w_fs, w_fi, w_counts;
    DevBuf w_voff, w_vsid, w_wslot; // compacted polygon vertex slots, their keys' table slots
    std::vector<double> mesh_verts;
    std::vector<int32_t> mesh_fs, mesh_fi;
    bool mesh_host = false; // the welded mesh has been copied into the vectors above

    ~am_engine()
    {
        if (own) cudaStreamSynchronize(own);
        release_run_buffers(); // pooled ones are freed in the order of a stream that still exists
        if (own) cudaStreamDestroy(own);
        if (h_ctl) cudaFreeHost(h_ctl);
        for (cudaEvent_t ev : {ev0, ev1, pa, pb})
            if (ev) cudaEventDestroy(ev);
        drop_graph();
    }

    RegionsDev regions() const
    {
        RegionsDev r;
        r.keys = keys.as<uint32_t>();
        r.hash = hash.as<uint64_t>();
        r.mid = mid.p;
        r.start = start.as<int32_t>();
        r.nv = nv.as<int32_t>();
        r.status = status.as<int8_t>();
        r.verts = verts.p;
        r.edges = edges.as<int32_t>();
        r.cap = cap;
        return r;
    }
    HashDev hashdev() const { return HashDev{table.as<unsigned long long>(), hcap - 1}; }
    // the region store, the table and the wave buffers go back to the device
    // (the next run allocates them afresh); the engine keeps no result
    void release_run_buffers()
    {
        drop_graph();
        for (DevBuf *b : {&keys, &hash, &mid, &start, &nv, &status, &verts, &edges, &table, &cons, &eq, &rec, &blocksum})
            b->reset();
        cap = 0;
        hcap = 0;
        chunk_cap = 0;
        num_regions = 0;
    }

    void ensure_regions(long long need)
    {
        if (need <= cap) return;
        long long nc = std::max<long long>(need, cap ? cap * 2 : (long long)1 << 16);
        const long long keep = num_regions;
        AM_CUDA(keys.grow(sizeof(uint32_t) * (size_t)W * nc, sizeof(uint32_t) * (size_t)W * keep, st));
        AM_CUDA(hash.grow(sizeof(uint64_t) * nc, sizeof(uint64_t) * keep, st));
        AM_CUDA(mid.grow(ts * 4 * nc, ts * 4 * keep, st));
        AM_CUDA(start.grow(sizeof(int32_t) * nc, sizeof(int32_t) * keep, st));
        AM_CUDA(nv.grow(sizeof(int32_t) * nc, sizeof(int32_t) * keep, st));
        AM_CUDA(status.grow(sizeof(int8_t) * nc, sizeof(int8_t) * keep, st));
        AM_CUDA(verts.grow(ts * 3 * kVMax * nc, ts * 3 * kVMax * keep, st));
        AM_CUDA(edges.grow(sizeof(int32_t) * kVMax * nc, sizeof(int32_t) * kVMax * keep, st));
        cap = nc;
    }

    // keep the load factor of the region table <= 1/2; with a fixed size
    // (AM_OPT_TABLE_SLOTS) the table never grows, and a run that outgrows it
    // ends with AM_ERR_TABLE_FULL when an insert reaches the probe bound
    void ensure_table(long long entries, bool rehash)
    {
        unsigned long long need = 1;
        if (table_slots > 0) {
            while (need < (unsigned long long)table_slots) need <<= 1;
            if (need == hcap) return;
            rehash = rehash && need > hcap;
        } else {
            while (need < (unsigned long long)std::max<long long>(entries, 1) * 2ull) need <<= 1;
            need = std::max<unsigned long long>(need, 1ull << 16);
            if (need <= hcap) return;
        }
        AM_CUDA(table.reserve(sizeof(unsigned long long) * need, st));
        hcap = need;
        AM_CUDA(cudaMemsetAsync(table.p, 0xff, sizeof(unsigned long long) * need, st));
        if (rehash && num_regions > 0) {
            launch_rehash(regions(), num_regions, hashdev(), d_err.as<int>(), st);
            AM_CUDA(cudaGetLastError());
        }
    }

    void ensure_chunk(int count)
    {
        if (count <= chunk_cap) return;
        AM_CUDA(cons.alloc(tc * 4 * (size_t)ALLP * count, st));
        AM_CUDA(eq.alloc(tc * 4 * (size_t)count, st));
        AM_CUDA(rec.alloc(sizeof(int32_t) * (size_t)kVMax * count, st));
        AM_CUDA(blocksum.alloc(sizeof(int) * ((size_t)count * kVMax / 1024 + 6), st));
        chunk_cap = count;
    }

    int default_chunk() const
    {
        if (chunk_opt > 0) return (int)std::min<int64_t>(chunk_opt, (int64_t)(0x7fffffff / std::max(ALL, 1)));
        // ~2 GiB of constraint rows per wave; a full wave of the tensor-core
        // composition is a whole number of rounds of one tile per SM (a
        // partly filled last round idles the other SMs)
        const size_t per = tc * 4 * (size_t)ALLP;
        long long c = (long long)((2ull << 30) / std::max<size_t>(per, 1));
        c = std::max<long long>(1024, std::min<long long>(c, 1 << 19));
        c = std::min<long long>(c, 0x7fffffff / std::max(ALL, 1));
        if (prec == kMixed && tcnet.ncols_max >= 16) {
            const long long round = (long long)device_sms() * (tcnet.ncols_max / 4);
            if (c > round) c = c / round * round;
        }
        return (int)c;
    }

    // one copy of (tail, error bits) after the work queued so far; throws on errors
    long long poll(size_t bytes = 16)
    {
        AM_CUDA(cudaMemcpyAsync(h_ctl, d_tail.p, bytes, cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        raise_device_errors(h_ctl->err);
        return h_ctl->tail;
    }
    // the control block's error bits as a status (the first that applies)
    static void raise_device_errors(int e)
    {
        if (e & kErrNonFinite)
            throw Failure{AM_ERR_INVALID_ARGUMENT, "weights, biases, transforms or extra constraints hold NaN or infinity"};
        if (e & kErrWait)
            throw Failure{AM_ERR_CUDA, "device wait limit reached: a bounded barrier wait (tensor-core pipeline or "
                                       "row copy) ran out, and the run's results are not valid"};
        if (e & kErrTableFull) throw Failure{AM_ERR_TABLE_FULL, "hash probe bound reached"};
        if (e & kErrCapacity) throw Failure{AM_ERR_CAPACITY, "region store capacity exceeded"};
    }
    WaveCtl *ctl() const { return (WaveCtl *)d_tail.p; }
    unsigned long long *fp64_counter() const
    {
        return (unsigned long long *)((char *)d_tail.p + kStatsOff) + kFp64Slot;
    }

    void drop_graph()
    {
        if (wexec) cudaGraphExecDestroy(wexec);
        if (wgraph) cudaGraphDestroy(wgraph);
        wexec = nullptr;
        wgraph = nullptr;
        wsig.clear();
    }

    // Run every remaining wave with one graph launch: one wave --
    // composition, polygons, append, step -- is captured as the body of a
    // conditional while node.  The kernels read the wave's range from the
    // control block, so the captured launches serve every wave, and the
    // instantiated graph is reused by later calls while the parameters it
    // captured (buffers, network layout, iso) are unchanged.
    void run_wave_graph(int prec, const NetDev &net, double iso, const Tolerances &tol, int chunk)
    {
        const RegionsDev reg = regions();
        const HashDev hs = hashdev();
        std::vector<unsigned char> sig;
        auto add = [&](const void *p, size_t n) {
            sig.insert(sig.end(), (const unsigned char *)p, (const unsigned char *)p + n);
        };
        const void *bufs[6] = {cons.p, eq.p, rec.p, blocksum.p, d_tail.p, (const void *)blocksum.bytes};
        add(&prec, sizeof(prec));
        add(&chunk, sizeof(chunk));
        add(&face_warps, sizeof(face_warps));
        add(&prune, sizeof(prune));
        add(&iso, sizeof(iso));
        add(&tol, sizeof(tol));
        add(&net, sizeof(net));
        if (prec == kMixed) add(&tcnet, sizeof(tcnet));
        add(&reg, sizeof(reg));
        add(&hs, sizeof(hs));
        add(bufs, sizeof(bufs));
        if (!wexec || sig != wsig) {
            drop_graph();
            try {
                AM_CUDA(cudaGraphCreate(&wgraph, 0));
                cudaGraphConditionalHandle cond;
                AM_CUDA(cudaGraphConditionalHandleCreate(&cond, wgraph, 1, cudaGraphCondAssignDefault));
                cudaGraphNodeParams np = {};
                np.type = cudaGraphNodeTypeConditional;
                np.conditional.handle = cond;
                np.conditional.type = cudaGraphCondTypeWhile;
                np.conditional.size = 1;
                cudaGraphNode_t node;
                AM_CUDA(cudaGraphAddNode(&node, wgraph, nullptr, nullptr, 0, &np));
                cudaGraph_t body = np.conditional.phGraph_out[0];
                AM_CUDA(cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
                ChunkDev ch;
                ch.head = 0;
                ch.count = chunk;
                ch.cons = cons.p;
                ch.eq = eq.p;
                ch.rec = rec.as<int32_t>();
                ch.ctl = ctl();
                if (prec == kMixed)
                    launch_compose_tc(net, tcnet, reg, ch, iso, d_err.as<int>(), st);
                else
                    launch_compose(prec, net, reg, ch, iso, st);
                launch_polygon(prec, net, reg, ch, hs, tol, face_warps, prune, fp64_counter(), d_err.as<int>(), st);
                launch_append(0, prec, net, reg, ch, hs, nullptr, nullptr, nullptr, chunk * kVMax,
                              d_tail.as<long long>(), blocksum.as<int>(), (int)(blocksum.bytes / sizeof(int)),
                              d_err.as<int>(), st);
                launch_wave_step(ctl(), cond, st);
                cudaGraph_t captured = nullptr;
                AM_CUDA(cudaStreamEndCapture(st, &captured));
                AM_CUDA(cudaGraphInstantiate(&wexec, wgraph, 0));
            } catch (...) {
                cudaStreamCaptureStatus cs;
                if (cudaStreamIsCapturing(st, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
                    cudaGraph_t g2 = nullptr;
                    cudaStreamEndCapture(st, &g2);
                }
                drop_graph();
                throw;
            }
            wsig.swap(sig);
        }
        AM_CUDA(cudaGraphLaunch(wexec, st));
    }
    void check_err() { poll(); }
};

namespace {

template <class F>
int guarded(am_engine *e, F &&f)
{
    try {
        f();
        return AM_OK;
    } catch (const Failure &x) {
        if (e) e->last_error = x.msg;
        return x.code;
    } catch (const std::bad_alloc &) {
        if (e) e->last_error = "host allocation failed";
        return AM_ERR_OUT_OF_MEMORY;
    }
}

int size_of_prec(int prec) { return prec == kFloat64 ? 8 : 4; }

} // namespace

// A run in phases, so that am_run_batch can interleave networks: begin
// (network upload, seed regions), the wave loop (graph-driven: launch, then
// poll; or host-driven), end (statistics).
struct RunArgs {
    const void *const *weights, *const *biases;
    const uint8_t *states;
    const void *points;
    int num_points;
    const void *const *arc_tm;
    const int32_t *arc_tm_shapes;
    int num_arc_tm;
    const void *w_extra, *b_extra;
    double iso;
    int flip_insideout;
    void *stream;
};

void run_begin(am_engine *e, const RunArgs &a)
{
    const void *const *weights = a.weights;
    const void *const *biases = a.biases;
    const uint8_t *states = a.states;
    const void *points = a.points;
    const int num_points = a.num_points;
    const void *const *arc_tm = a.arc_tm;
    const int32_t *arc_tm_shapes = a.arc_tm_shapes;
    const int num_arc_tm = a.num_arc_tm;
    const void *w_extra = a.w_extra, *b_extra = a.b_extra;
    const double iso = a.iso;
    void *stream = a.stream;
    e->ensure_events();
    e->st = stream ? (cudaStream_t)stream : e->own;
    cudaStream_t st = e->st;
    const int prec = e->prec;
    const size_t tc = e->tc, ts = e->ts;
    AM_CHECK(weights && biases, "weights / biases are NULL");
    AM_CHECK(states && points && num_points >= 1, "states / points are empty"); // cuam.cpp:142
    AM_CHECK(e->E == 0 || (w_extra && b_extra), "extra constraints are NULL");
    // arc_tm shapes, cuam.cpp:160-173
    for (int i = 0; i + 1 < e->n_lin; ++i) {
        const int *row = e->arc.data() + (size_t)i * e->arc_cols;
        for (int c = 0; c < row[0]; ++c) {
            const int from = row[1 + 2 * c], t = row[2 + 2 * c];
            AM_CHECK(t >= 0 && t < num_arc_tm && arc_tm_shapes, "arc_table refers to a missing transform");
            const int h = arc_tm_shapes[2 * t], w = arc_tm_shapes[2 * t + 1];
            if (h || w) {
                AM_CHECK(h == e->nodes[i + 2], "transform rows must match the target width");
                AM_CHECK(w == e->nodes[from], "transform columns must match the source width");
            } else {
                AM_CHECK(e->nodes[from] == e->nodes[i + 2], "identity connection between different widths");
            }
        }
    }


    // ---------------------------------------------------------- network
    NetDev &net = e->net;
    memset(&net, 0, sizeof(net));
    net.n_lin = e->n_lin;
    net.N = e->N;
    net.E = e->E;
    net.ALL = e->ALL;
    net.ALLP = e->ALLP;
    net.W = e->W;
    for (int i = 0; i <= e->n_lin; ++i) net.nodes[i] = e->nodes[i];
    net.hoff[1] = 0;
    for (int h = 1; h < e->n_lin; ++h) net.hoff[h + 1] = net.hoff[h] + e->nodes[h];
    for (int i = 0; i < e->n_lin; ++i) {
        const int M = e->nodes[i + 1], K = e->nodes[i];
        AM_CHECK(weights[i] && biases[i], "a weight / bias pointer is NULL");
        upload(e->bias[i], biases[i], tc * M, st);
        net.bias[i] = e->bias[i].p;
        if (i == 0) {
            upload(e->w0, weights[0], tc * (size_t)M * 3, st);
            net.W0 = e->w0.p;
        } else {
            const int Mp = (M + 3) / 4 * 4;
            upload(e->scratch, weights[i], tc * (size_t)M * K, st);
            AM_CUDA(e->wt[i].reserve(tc * (size_t)K * Mp));
            launch_prepare_weights(prec == kFloat64 ? kFloat64 : kFloat32, e->scratch.p, M, K, Mp, e->wt[i].p, st);
            net.Wt[i] = e->wt[i].p;
            net.Mp[i] = Mp;
        }
    }
    int ntm = 0;
    long long *tm_count = e->tm_count;
    for (int i = 1; i < e->n_lin; ++i) {
        const int *row = e->arc.data() + (size_t)(i - 1) * e->arc_cols;
        net.nskip[i] = row[0];
        for (int c = 0; c < row[0]; ++c) {
            const int from = row[1 + 2 * c], t = row[2 + 2 * c];
            SkipDev &sk = net.skip[i][c];
            sk.from = from;
            const int h = arc_tm_shapes[2 * t], w = arc_tm_shapes[2 * t + 1];
            if (h == 0 && w == 0) {
                sk.kind = 0;
                sk.tmt = nullptr;
                sk.Mp = 0;
            } else {
                AM_CHECK(ntm < 64, "too many transform matrices");
                const int Mp = (h + 3) / 4 * 4;
                upload(e->scratch, arc_tm[t], tc * (size_t)h * w, st);
                AM_CUDA(e->tmt[ntm].reserve(tc * (size_t)w * Mp));
                launch_prepare_weights(prec == kFloat64 ? kFloat64 : kFloat32, e->scratch.p, h, w, Mp,
                                       e->tmt[ntm].p, st);
                sk.kind = 1;
                sk.tmt = e->tmt[ntm].p;
                sk.Mp = Mp;
                tm_count[ntm] = (long long)w * Mp;
                ntm++;
            }
        }
    }
    e->ntm = ntm;
    if (e->E) {
        upload(e->wext, w_extra, tc * 3 * (size_t)e->E, st);
        upload(e->bext, b_extra, tc * (size_t)e->E, st);
    }
    net.w_extra = e->wext.p;
    net.b_extra = e->bext.p;
    {
        // every parameter finite (checked on the device copies, one launch;
        // decoded as AM_ERR_INVALID_ARGUMENT by the first poll)
        FiniteList fl{};
        auto add = [&](const void *p, long long n) {
            if (p && n > 0 && fl.count < 64) {
                fl.p[fl.count] = p;
                fl.n[fl.count++] = n;
            }
        };
        AM_CUDA(cudaMemsetAsync(e->d_err.p, 0, sizeof(int), st));
        for (int i = 0; i < e->n_lin; ++i) add(e->bias[i].p, e->nodes[i + 1]);
        add(e->w0.p, 3ll * e->nodes[1]);
        for (int i = 1; i < e->n_lin; ++i) add(e->wt[i].p, (long long)e->nodes[i] * net.Mp[i]);
        for (int t = 0; t < ntm; ++t) add(e->tmt[t].p, tm_count[t]);
        if (e->E) {
            add(e->wext.p, 3ll * e->E);
            add(e->bext.p, e->E);
        }
        launch_check_finite(prec == kFloat64 ? kFloat64 : kFloat32, fl, e->d_err.as<int>(), st);
    }
    if (prec == kMixed) {
        // three bf16 terms per weight, stored as 128 x 64 shared-memory block images
        TcNet &tc = e->tcnet;
        memset(&tc, 0, sizeof(tc));
        tc.mtiles_max = 1;
        tc.mgroups = 1;
        auto split = [&](DevBuf &buf, const void *src_fp32, int M, int K, TcMat &m) {
            const int Mp = (M + 127) / 128 * 128, Kp = (K + 63) / 64 * 64;
            upload(e->scratch, src_fp32, sizeof(float) * (size_t)M * K, st);
            AM_CUDA(buf.reserve((size_t)(Mp / 128) * (Kp / 64) * kWBlockBytes));
            launch_pack_weights(e->scratch.as<float>(), M, K, Mp, Kp, buf.p, st);
            m.blocks = (const uint8_t *)buf.p;
            m.Mp = Mp;
            m.Kp = Kp;
            tc.kp_max = std::max(tc.kp_max, Kp);
            tc.mtiles_max = std::max(tc.mtiles_max, Mp / 128);
        };
        for (int i = 1; i <= e->n_lin - 2; ++i) {
            split(e->tc_lin[i], weights[i], e->nodes[i + 1], e->nodes[i], tc.lin[i]);
            const int *row = e->arc.data() + (size_t)(i - 1) * e->arc_cols;
            for (int c = 0; c < row[0]; ++c) {
                const int from = row[1 + 2 * c], t = row[2 + 2 * c];
                const int h = arc_tm_shapes[2 * t], w = arc_tm_shapes[2 * t + 1];
                if ((h || w) && from >= 1) split(e->tc_skip[i][c], arc_tm[t], h, w, tc.skip[i][c]);
            }
        }
        // the operand also holds hidden layer 1 and the last hidden layer
        tc.kp_max = std::max(tc.kp_max, (e->nodes[1] + 63) / 64 * 64);
        tc.kp_max = std::max(tc.kp_max, (e->nodes[e->n_lin - 1] + 63) / 64 * 64);
        // widest tile: three operand terms (3 x ncols x kp_max x 2 bytes)
        // beside two weight blocks in flight (one if that leaves no room),
        // two accumulators (main + correction) per M tile in 512 TMEM columns
        const size_t smem_cap = 227u * 1024u;
        // preference: MN-major operand (whole 64-column atoms), two weight
        // stages, then one; then the K-major operand (any 16 columns)
        tc.ncols_max = 0;
        tc.n1 = e->nodes[1];
        tc.k_last = e->nodes[e->n_lin - 1];
        for (int mn = 1; mn >= 0 && tc.ncols_max < 16; --mn)
            for (tc.nstage = 2; tc.nstage >= 1; --tc.nstage) {
                const long long room = (long long)smem_cap - 1024 - (long long)tc.nstage * kWBlockBytes -
                                       64ll * (e->W | 1) * 4 - 16ll * tc.n1 - 4ll * tc.k_last - 16 - 512 * 16;
                long long c = std::max<long long>(0, room) / (6ll * tc.kp_max);
                if (mn) c = c / 64 * 64;
                int ncols = (int)std::min<long long>(c, 256);
                ncols = std::min(ncols, 256 / tc.mtiles_max) / 16 * 16;
                tc.ncols_max = ncols;
                tc.mn = mn;
                if (ncols >= 16) break;
            }
        // streamed operand (wide layers): two 64-deep operand blocks, so the
        // tile is as wide as TMEM allows; taken when that is wider
        // (the widest tile first, then the most weight stages in flight)
        // With mgroups > 1 a layer's M tiles are multiplied in that many
        // passes, each with its own accumulators, so that the tile can be
        // wider than two accumulators per M tile of the widest layer allow
        // (the operand is rebuilt once per pass).
        auto streamed_tile = [&](int mgroups) {
            TcNet ts = tc;
            ts.streamed = 1;
            ts.mgroups = mgroups;
            ts.ncols_max = 0;
            const int mper = (ts.mtiles_max + mgroups - 1) / mgroups;
            for (int mn = 1; mn >= 0 && ts.ncols_max < 16; --mn) {
                ts.mn = mn;
                for (int ncols = std::min(256, 256 / mper) / 16 * 16; ncols >= 16 && ts.ncols_max < 16; ncols -= 16)
                    for (int ns = 3; ns >= 1; --ns) {
                        ts.ncols_max = ncols;
                        ts.nstage = ns;
                        if (tc_smem_bytes(ts, ncols, e->W) <= smem_cap) break;
                        ts.ncols_max = 0;
                    }
            }
            return ts;
        };
        TcNet ts = streamed_tile(1);
        if (tc.mtiles_max >= 2 && e->compose_tile != 2) {
            // two passes pay for rebuilding the operand and a second epilogue
            // per layer: automatically only for twice the tile width with two
            // weight stages or more (measured on GB300: 3-[512]x8-1 faster
            // with 128 columns in two passes than 64 in one, 3-[256]x6-1
            // slower with a wider two-pass tile than 128 columns in one)
            const TcNet t2 = streamed_tile(2);
            if (e->compose_tile == 3 || (t2.ncols_max >= 2 * ts.ncols_max && t2.nstage >= 2)) ts = t2;
        }
        const bool want_streamed = e->compose_tile >= 2 ||
                                   (e->compose_tile == 0 && tc.kp_max >= 256 && ts.ncols_max > tc.ncols_max);
        if (ts.ncols_max >= 16 && (want_streamed || tc.ncols_max < 16)) tc = ts;
        AM_CHECK(e->compose_tile != 1 || !tc.streamed, "resident operand tile does not fit");
        AM_CHECK(tc.nstage >= 1 && tc.ncols_max >= 16, "layer widths too large for the tensor-core composition tile");
        AM_CHECK(tc_smem_bytes(tc, tc.ncols_max, e->W) <= smem_cap,
                 "tensor-core composition tile exceeds shared memory");
    }
    AM_CUDA(cudaGetLastError());

    // ---------------------------------------------------------- seeds
    const int S = num_points;
    upload(e->s_states, states, (size_t)S * e->N, st);
    {
        // seed points in the solve precision
        std::vector<double> pd(3 * (size_t)S);
        std::vector<unsigned char> raw(tc * 3 * (size_t)S);
        to_host(raw.data(), points, raw.size(), st);
        AM_CUDA(cudaStreamSynchronize(st));
        for (size_t q = 0; q < 3 * (size_t)S; ++q)
            pd[q] = tc == 8 ? ((const double *)raw.data())[q] : (double)((const float *)raw.data())[q];
        if (ts == 8) {
            upload(e->s_pts, pd.data(), sizeof(double) * pd.size(), st);
        } else {
            std::vector<float> pf(pd.begin(), pd.end());
            upload(e->s_pts, pf.data(), sizeof(float) * pf.size(), st);
        }
        AM_CUDA(cudaStreamSynchronize(st));
    }
    AM_CUDA(e->s_keys.reserve(sizeof(uint32_t) * (size_t)S * e->W));
    AM_CUDA(e->s_hash.reserve(sizeof(uint64_t) * (size_t)S));
    AM_CUDA(e->s_rec.reserve(sizeof(int32_t) * (size_t)S));

    e->num_regions = 0;
    e->hcap = 0;
    e->stats = am_stats{};
    AM_CUDA(cudaMemsetAsync(e->d_tail.p, 0, sizeof(long long), st));
    AM_CUDA(cudaMemsetAsync(e->fp64_counter(), 0, sizeof(unsigned long long), st));
    const int chunk = e->default_chunk();
    e->ensure_chunk(std::min(chunk, std::max(S, 1024)));
    // the first stores hold the seeds' children of a first wave (a batch
    // member's, or a small network's, grow on demand from there)
    const long long first_wave = std::min<long long>(chunk, e->lean ? 4ll * S + 1024 : std::max(4ll * S + 1024, 65536ll));
    e->ensure_regions(std::max<long long>(S, 1) + first_wave * kVMax);
    e->ensure_table((long long)S + first_wave * kVMax, false);
    AM_CUDA(e->blocksum.grow(sizeof(int) * ((size_t)S / 1024 + 6), 0, st));
    AM_CUDA(cudaStreamSynchronize(st));

    e->run.launches = 0;
    AM_CUDA(cudaEventRecord(e->ev0, st));
    launch_seed_pack(e->s_states.as<uint8_t>(), S, e->N, e->W, e->s_keys.as<uint32_t>(), e->s_hash.as<uint64_t>(), st);
    launch_seed_insert(e->s_keys.as<uint32_t>(), e->s_hash.as<uint64_t>(), S, e->W, e->hashdev(),
                       e->s_rec.as<int32_t>(), e->d_err.as<int>(), st);
    {
        ChunkDev sc{};
        sc.rec = e->s_rec.as<int32_t>();
        launch_append(1, prec, net, e->regions(), sc, e->hashdev(), e->s_keys.as<uint32_t>(),
                      e->s_hash.as<uint64_t>(), e->s_pts.p, S, e->d_tail.as<long long>(), e->blocksum.as<int>(),
                      (int)(e->blocksum.bytes / sizeof(int)), e->d_err.as<int>(), st);
    }
    e->run.launches += 5; // + the parameter check
    AM_CUDA(cudaGetLastError());
    const long long tail = e->poll();
    e->num_regions = tail;
    e->stats.num_seeds = tail;
    if (e->inject_err) {
        // test hook: error bits as a kernel would leave them, for the wave
        // loop's error decoding to find
        e->h_ctl->err = e->inject_err;
        AM_CUDA(cudaMemcpyAsync(e->d_err.p, &e->h_ctl->err, sizeof(int), cudaMemcpyHostToDevice, st));
        AM_CUDA(cudaStreamSynchronize(st));
    }

    am_engine::Run &r = e->run;
    r.prec = prec;
    r.iso = iso;
    r.tol = prec == kFloat64 ? Tolerances{1e-20, 3e-14, 1e-12} : Tolerances{1e-12, 3e-7, 1e-6};
    r.chunk = chunk;
    r.head = 0;
    r.tail = tail;
    r.chunks = 0;
    r.t_comp = r.t_poly = r.t_front = 0;
    r.flip = a.flip_insideout != 0;
    r.lean = e->lean;
}

// graph-driven loop: one graph launch runs up to max_waves waves, until the
// queue is empty; it stops early when the next wave's children might not
// fit, and then resumes after the host grows the region store and the
// table.  The control block comes back to pinned memory behind the graph.
void run_graph_launch(am_engine *e, int max_waves)
{
    am_engine::Run &r = e->run;
    cudaStream_t st = e->st;
    // the largest wave of this launch: the chunk, or for a batch member the
    // queue's length rounded up to a power of two (at most the chunk), so
    // that many small networks do not each hold a full chunk of rows; the
    // loop stops when the queue outgrows it and the next launch grows it
    const long long pending = r.tail - r.head;
    int wave = r.chunk;
    if (r.lean) {
        long long w = std::max(e->chunk_cap, 1024);
        while (w < pending && w < r.chunk) w *= 2;
        wave = (int)std::min<long long>(w, r.chunk);
    }
    e->ensure_chunk(wave);
    const int count = (int)std::min<long long>(pending, wave);
    e->ensure_regions(r.tail + (long long)count * kVMax);
    e->ensure_table(std::max<long long>(r.tail + (long long)count * kVMax, e->cap), true);
    WaveCtl *h = e->h_ctl;
    h->head = r.head;
    h->count = count;
    h->waves = 0;
    h->limit = e->table_slots > 0 ? e->cap : std::min<long long>(e->cap, (long long)(e->hcap / 2));
    h->chunk_cap = wave;
    h->grow_at = wave < r.chunk ? (int)std::min<long long>(2ll * wave, INT_MAX) : INT_MAX;
    h->work = 0u;
    h->max_waves = max_waves;
    h->stop_tail = e->max_regions > 0 ? e->max_regions : LLONG_MAX;
    // tail and err stay as the device has them
    AM_CUDA(cudaMemcpyAsync((char *)e->d_tail.p + offsetof(WaveCtl, head), (char *)h + offsetof(WaveCtl, head),
                            sizeof(WaveCtl) - offsetof(WaveCtl, head), cudaMemcpyHostToDevice, st));
    e->run_wave_graph(r.prec, e->net, r.iso, r.tol, wave);
    AM_CUDA(cudaMemcpyAsync(h, e->d_tail.p, sizeof(WaveCtl), cudaMemcpyDeviceToHost, st));
}

// after the stream has reached the end of the launch: true while regions remain
bool run_graph_done(am_engine *e)
{
    am_engine::Run &r = e->run;
    const WaveCtl *h = e->h_ctl;
    am_engine::raise_device_errors(h->err);
    AM_CHECK(h->waves < kMaxWaves, "wave bound reached");
    r.tail = h->tail;
    r.chunks += h->waves;
    r.launches += 5ll * h->waves;
    r.head = h->head;
    e->num_regions = r.tail;
    if (e->over_limit(r.tail)) return false; // stop: the regions so far stay
    return r.head < r.tail;
}

// host-driven loop (phase timing, or AM_OPT_GRAPH = 0)
void run_host_loop(am_engine *e)
{
    am_engine::Run &run = e->run;
    cudaStream_t st = e->st;
    const int prec = run.prec;
    const NetDev &net = e->net;
    const double iso = run.iso;
    const Tolerances tol = run.tol;
    const int chunk = run.chunk;
    long long head = run.head, tail = run.tail, launches = run.launches;
    int chunks = run.chunks;
    double t_comp = 0, t_poly = 0, t_front = 0;
    cudaEvent_t pa = e->pa, pb = e->pb;
    while (head < tail) {
        const int count = (int)std::min<long long>(tail - head, chunk);
        e->ensure_chunk(count);
        e->ensure_regions(tail + (long long)count * kVMax);
        e->ensure_table(tail + (long long)count * kVMax, true);
        ChunkDev ch;
        ch.head = head;
        ch.count = count;
        ch.cons = e->cons.p;
        ch.eq = e->eq.p;
        ch.rec = e->rec.as<int32_t>();
        const RegionsDev reg = e->regions();
        const HashDev hs = e->hashdev();
        float ms = 0;
        if (e->phase_timing) AM_CUDA(cudaEventRecord(pa, st));
        if (prec == kMixed)
            launch_compose_tc(net, e->tcnet, reg, ch, iso, e->d_err.as<int>(), st);
        else
            launch_compose(prec, net, reg, ch, iso, st);
        if (e->phase_timing) {
            AM_CUDA(cudaEventRecord(pb, st));
            AM_CUDA(cudaEventSynchronize(pb));
            AM_CUDA(cudaEventElapsedTime(&ms, pa, pb));
            t_comp += ms;
            AM_CUDA(cudaEventRecord(pa, st));
        }
        launch_polygon(prec, net, reg, ch, hs, tol, e->face_warps, e->prune, e->fp64_counter(), e->d_err.as<int>(),
                       st);
        if (e->phase_timing) {
            AM_CUDA(cudaEventRecord(pb, st));
            AM_CUDA(cudaEventSynchronize(pb));
            AM_CUDA(cudaEventElapsedTime(&ms, pa, pb));
            t_poly += ms;
            AM_CUDA(cudaEventRecord(pa, st));
        }
        launch_append(0, prec, net, reg, ch, hs, nullptr, nullptr, nullptr, count * kVMax, e->d_tail.as<long long>(),
                      e->blocksum.as<int>(), (int)(e->blocksum.bytes / sizeof(int)), e->d_err.as<int>(), st);
        if (e->phase_timing) {
            AM_CUDA(cudaEventRecord(pb, st));
            AM_CUDA(cudaEventSynchronize(pb));
            AM_CUDA(cudaEventElapsedTime(&ms, pa, pb));
            t_front += ms;
        }
        launches += 4;
        AM_CUDA(cudaGetLastError());
        head += count;
        tail = e->poll();
        e->num_regions = tail;
        chunks++;
        if (e->over_limit(tail)) break;
    }
    run.head = head;
    run.tail = tail;
    run.launches = launches;
    run.chunks = chunks;
    run.t_comp = t_comp;
    run.t_poly = t_poly;
    run.t_front = t_front;
}

void run_end(am_engine *e)
{
    am_engine::Run &run = e->run;
    cudaStream_t st = e->st;
    const long long tail = run.tail;
    const int chunks = run.chunks;
    const long long launches = run.launches;
    const double t_comp = run.t_comp, t_poly = run.t_poly, t_front = run.t_front;
    const int flip_insideout = run.flip ? 1 : 0;
    const double iso = run.iso;
    cudaEvent_t ev0 = e->ev0, ev1 = e->ev1;
    AM_CUDA(cudaEventRecord(ev1, st));
    AM_CUDA(cudaEventSynchronize(ev1));
    float total = 0;
    AM_CUDA(cudaEventElapsedTime(&total, ev0, ev1));
    e->check_err();

    // statistics
    am_stats &sx = e->stats;
    sx.num_regions = tail;
    sx.chunks = chunks;
    sx.am_time_ms = total;
    sx.compose_ms = t_comp;
    sx.polygon_ms = t_poly;
    sx.frontier_ms = t_front;
    sx.kernel_launches = launches;
    {
        // face and status counts, reduced on the device (48 bytes come back)
        unsigned long long *d = (unsigned long long *)((char *)e->d_tail.p + kStatsOff);
        const unsigned long long *h = (const unsigned long long *)((const char *)e->h_ctl + kStatsOff);
        AM_CUDA(cudaMemsetAsync(d, 0, kStatsCount * sizeof(unsigned long long), st));
        launch_region_stats(e->nv.as<int32_t>(), e->status.as<int8_t>(), tail, d, st);
        AM_CUDA(cudaMemcpyAsync((char *)e->h_ctl + kStatsOff, d, (kStatsCount + 1) * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        sx.num_faces = (int64_t)h[0];
        sx.max_polygon_verts = (int32_t)h[1];
        sx.num_nostart = (int64_t)h[2 + kNoStart - 1];
        sx.num_open = (int64_t)h[2 + kOpen - 1];
        sx.num_truncated = (int64_t)h[2 + kTruncated - 1];
        sx.num_singular = (int64_t)h[2 + kSingular - 1];
        sx.num_fp64_walks = (int64_t)h[kFp64Slot];
    }
    e->flip = flip_insideout ? 1 : 0;
    e->iso = iso;
    e->has_am = true;
}

extern "C" {

const char *am_strerror(int s)
{
    switch (s) {
    case AM_OK: return "ok";
    case AM_ERR_INVALID_ARGUMENT: return "invalid argument";
    case AM_ERR_NOT_INITIALIZED: return "engine not initialised";
    case AM_ERR_CUDA: return "CUDA error";
    case AM_ERR_OUT_OF_MEMORY: return "out of memory";
    case AM_ERR_TABLE_FULL: return "region hash table full";
    case AM_ERR_NO_RESULT: return "no result: run AnalyticMarching (and CombineMesh) first";
    case AM_ERR_IO: return "I/O error";
    case AM_ERR_CAPACITY: return "region store capacity exceeded";
    default: return "unknown status";
    }
}

const char *am_last_error(const am_engine *e) { return e ? e->last_error.c_str() : "null engine"; }

int am_vert_capacity(void) { return kVMax; }

int am_init(am_engine **out, const char *float_type, const int32_t *nodesnum, int num_nodes, const int32_t *arc_table,
            int arc_rows, int arc_cols, int num_extra_constraints)
{
    if (!out) return AM_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    std::unique_ptr<am_engine> e(new am_engine());
    int rc = guarded(e.get(), [&] {
        AM_CHECK(float_type, "float_type is NULL");
        const std::string ft(float_type);
        AM_CHECK(ft == "float32" || ft == "float64" || ft == "mixed", "float_type is either float32, float64 or mixed");
        e->prec = ft == "float64" ? kFloat64 : (ft == "mixed" ? kMixed : kFloat32);
        e->tc = size_of_prec(e->prec == kMixed ? kFloat32 : e->prec);
        e->ts = e->prec == kFloat32 ? 4 : 8;
        // cuam.cpp:69-86
        AM_CHECK(nodesnum && num_nodes >= 3, "nodesnum needs at least 3 entries");
        AM_CHECK(nodesnum[0] == 3, "nodesnum[0] must be 3");
        AM_CHECK(nodesnum[num_nodes - 1] == 1, "nodesnum[-1] must be 1");
        AM_CHECK(num_nodes - 1 <= kMaxLayers, "too many layers");
        AM_CHECK(arc_rows == num_nodes - 2, "arc_table must have len(nodesnum) - 2 rows");
        AM_CHECK(arc_cols >= 1 && (arc_cols + 1) % 2 == 0, "arc_table width must be odd");
        AM_CHECK(num_extra_constraints >= 0, "num_extra_constraints must be >= 0");
        AM_CHECK(arc_table || arc_rows == 0, "arc_table is NULL");
        for (int i = 0; i < arc_rows; ++i) {
            const int cnt = arc_table[(size_t)i * arc_cols];
            AM_CHECK(cnt >= 0 && 1 + 2 * cnt <= arc_cols, "arc_table row has more connections than columns");
            AM_CHECK(cnt <= kMaxSkips, "too many connections into one layer");
            for (int c = 0; c < cnt; ++c) {
                const int from = arc_table[(size_t)i * arc_cols + 1 + 2 * c];
                AM_CHECK(from >= 0 && from <= i + 1, "arc_table source must precede the target layer");
            }
        }
        for (int i = 0; i < num_nodes; ++i) AM_CHECK(nodesnum[i] > 0, "layer widths must be positive");
        e->nodes.assign(nodesnum, nodesnum + num_nodes);
        e->arc.assign(arc_table, arc_table + (size_t)arc_rows * arc_cols);
        e->arc_cols = arc_cols;
        e->n_lin = num_nodes - 1;
        e->N = 0;
        for (int i = 1; i < num_nodes - 1; ++i) e->N += nodesnum[i];
        e->E = num_extra_constraints;
        e->ALL = e->N + e->E;
        e->ALLP = (e->ALL + 7) / 8 * 8;
        e->W = (e->N + 31) / 32;
        AM_CHECK((size_t)e->ALLP * 4 * (e->prec == kFloat64 ? 8 : 4) <= 200u * 1024u,
                 "too many constraint rows for one face (sum of hidden widths + extra constraints)");
        AM_CUDA(cudaStreamCreateWithFlags(&e->own, cudaStreamNonBlocking));
        e->st = e->own;
        AM_CUDA(e->d_tail.alloc(kCtlBytes));
        AM_CUDA(cudaMemset(e->d_tail.p, 0, kCtlBytes));
        e->d_err.p = &((WaveCtl *)e->d_tail.p)->err;
        AM_CUDA(cudaHostAlloc((void **)&e->h_ctl, kCtlBytes, cudaHostAllocDefault));
        memset(e->h_ctl, 0, kCtlBytes);
    });
    if (rc == AM_OK) *out = e.release();
    return rc;
}

int am_set_option(am_engine *e, int option, int64_t value)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (option == AM_OPT_CHUNK) {
        if (value < 0) return AM_ERR_INVALID_ARGUMENT;
        e->chunk_opt = value;
        return AM_OK;
    }
    if (option == AM_OPT_PHASE_TIMING) {
        e->phase_timing = value != 0;
        return AM_OK;
    }
    if (option == AM_OPT_WELD) {
        if (value != 0 && value != 1) return AM_ERR_INVALID_ARGUMENT;
        e->weld_mode = (int)value;
        return AM_OK;
    }
    if (option == AM_OPT_GRAPH) {
        e->use_graph = value != 0;
        return AM_OK;
    }
    if (option == AM_OPT_MAX_REGIONS) {
        if (value < 0) return AM_ERR_INVALID_ARGUMENT;
        e->max_regions = value;
        return AM_OK;
    }
    if (option == AM_OPT_FACE_WARPS) {
        if (value != 0 && value != 1 && value != 2 && value != 4 && value != 8) return AM_ERR_INVALID_ARGUMENT;
        e->face_warps = (int)value;
        return AM_OK;
    }
    if (option == AM_OPT_COMPOSE_TILE) {
        if (value < 0 || value > 3) return AM_ERR_INVALID_ARGUMENT;
        e->compose_tile = (int)value;
        return AM_OK;
    }
    if (option == AM_OPT_TABLE_SLOTS) {
        if (value < 0 || value > (int64_t(1) << 40)) return AM_ERR_INVALID_ARGUMENT;
        e->table_slots = value;
        e->hcap = 0; // the next run sizes the table afresh
        return AM_OK;
    }
    if (option == AM_OPT_PRUNE_ROWS) {
        if (value != 0 && value != 1) return AM_ERR_INVALID_ARGUMENT;
        e->prune = (int)value;
        return AM_OK;
    }
    if (option == AM_OPT_INJECT_ERROR) {
        if (value < 0 || value > (kErrTableFull | kErrWait | kErrCapacity | kErrNonFinite)) return AM_ERR_INVALID_ARGUMENT;
        e->inject_err = (int)value;
        return AM_OK;
    }
    return AM_ERR_INVALID_ARGUMENT;
}

int am_analytic_marching(am_engine *e, const void *const *weights, const void *const *biases, const uint8_t *states,
                         const void *points, int num_points, const void *const *arc_tm, const int32_t *arc_tm_shapes,
                         int num_arc_tm, const void *w_extra, const void *b_extra, double iso, int flip_insideout,
                         void *stream)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    e->has_am = false;
    e->has_mesh = false;
    const RunArgs a{weights, biases, states, points, num_points, arc_tm, arc_tm_shapes, num_arc_tm,
                    w_extra, b_extra, iso, flip_insideout, stream};
    e->limit_hit = false;
    return guarded(e, [&] {
        run_begin(e, a);
        if (e->use_graph && !e->phase_timing) {
            while (e->run.head < e->run.tail) {
                run_graph_launch(e, kMaxWaves);
                AM_CUDA(cudaStreamSynchronize(e->st));
                if (!run_graph_done(e)) break;
            }
        } else {
            run_host_loop(e);
        }
        run_end(e);
        if (e->limit_hit) // the results so far are kept (has_am) and reported as a stop
            throw Failure{AM_ERR_CAPACITY,
                          "region limit reached: stopped at " + std::to_string(e->run.tail) + " regions"};
    });
}

// Autotuner: the composition tile (resident or streamed operand, mixed form)
// and the warps per face polygon, chosen for a network architecture by
// marching a sample of it (the first sample_regions regions, the region limit
// of AM_OPT_MAX_REGIONS) once per candidate with per-phase device timing,
// after one untimed pass over the candidates (first launches load modules).
// Every candidate produces the same regions (the options change the work
// split, not the result), so the samples time the same waves.  The choice
// is kept per architecture for the process.
namespace {
std::mutex g_tune_mu;
std::map<std::vector<int64_t>, std::pair<int, int>> g_tune;
} // namespace

int am_autotune(am_engine *e, const am_run_args *x, int64_t sample_regions, int32_t *chosen)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!x || sample_regions < 1) return AM_ERR_INVALID_ARGUMENT;
    std::vector<int64_t> key = {e->prec, e->E, sample_regions};
    key.insert(key.end(), e->nodes.begin(), e->nodes.end());
    key.insert(key.end(), e->arc.begin(), e->arc.end());
    for (int t = 0; t < x->num_arc_tm && x->arc_tm_shapes; ++t) {
        key.push_back(x->arc_tm_shapes[2 * t]);
        key.push_back(x->arc_tm_shapes[2 * t + 1]);
    }
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) {
            e->compose_tile = it->second.first;
            e->face_warps = it->second.second;
            if (chosen) chosen[0] = e->compose_tile, chosen[1] = e->face_warps;
            return AM_OK;
        }
    }
    const RunArgs a{x->weights, x->biases, x->states, x->points, x->num_points, x->arc_tm, x->arc_tm_shapes,
                    x->num_arc_tm, x->w_extra, x->b_extra, x->iso, x->flip_insideout, nullptr};
    const long long keep_max = e->max_regions;
    const bool keep_pt = e->phase_timing;
    const int keep_ct = e->compose_tile, keep_fw = e->face_warps;
    int last_rc = AM_OK;
    auto sample = [&](int ct, int fw, double &comp, double &poly) {
        e->compose_tile = ct;
        e->face_warps = fw;
        e->max_regions = sample_regions;
        e->phase_timing = true;
        e->has_am = false;
        e->has_mesh = false;
        e->limit_hit = false;
        e->lean = true; // stores sized to the sample, not to a full chunk
        const int rc = guarded(e, [&] {
            run_begin(e, a);
            run_host_loop(e);
            run_end(e);
        });
        e->lean = false;
        if (rc != AM_OK) last_rc = rc;
        comp = e->stats.compose_ms;
        poly = e->stats.polygon_ms;
        return rc == AM_OK;
    };
    std::vector<int> cts = {0};
    if (e->prec == kMixed) cts = {1, 2, 3};
    const int fws[] = {1, 2, 4, 8};
    double c = 0, p = 0;
    for (int ct : cts) sample(ct, 0, c, p); // untimed pass
    for (int fw : fws) sample(0, fw, c, p);
    int best_ct = -1, best_fw = -1;
    double best = 1e300;
    for (int ct : cts)
        if (sample(ct, 0, c, p) && c < best) best = c, best_ct = ct;
    best = 1e300;
    if (best_ct >= 0)
        for (int fw : fws)
            if (sample(best_ct, fw, c, p) && p < best) best = p, best_fw = fw;
    e->max_regions = keep_max;
    e->phase_timing = keep_pt;
    e->has_am = false; // the samples are not a result
    e->has_mesh = false;
    e->limit_hit = false;
    // many engines are tuned before a batch: none keeps its sample's stores
    guarded(e, [&] {
        AM_CUDA(cudaStreamSynchronize(e->st));
        e->release_run_buffers();
    });
    if (best_ct < 0 || best_fw < 0) {
        e->compose_tile = keep_ct;
        e->face_warps = keep_fw;
        return last_rc != AM_OK ? last_rc : AM_ERR_CUDA;
    }
    e->compose_tile = best_ct;
    e->face_warps = best_fw;
    {
        std::lock_guard<std::mutex> lock(g_tune_mu);
        g_tune[key] = {best_ct, best_fw};
    }
    if (chosen) chosen[0] = best_ct, chosen[1] = best_fw;
    return AM_OK;
}

int am_run_batch(am_engine *const *engines, const am_run_args *args, int count, double *wall_ms)
{
    if (!engines || !args || count < 1) return AM_ERR_INVALID_ARGUMENT;
    for (int i = 0; i < count; ++i) {
        if (!engines[i]) return AM_ERR_NOT_INITIALIZED;
        for (int j = 0; j < i; ++j)
            if (engines[j] == engines[i]) return AM_ERR_INVALID_ARGUMENT; // one run per engine
    }
    DeferFrees defer;
    std::vector<char> active((size_t)count, 0);
    // begin each network and start its wave loop right away, on its own
    // stream, with full grids: a network whose waves fill the GPU runs as
    // fast as alone, the waves of smaller ones fill the gaps
    for (int i = 0; i < count; ++i) {
        am_engine *e = engines[i];
        const am_run_args &x = args[i];
        e->has_am = false;
        e->has_mesh = false;
        e->lean = true; // stores start small and grow on demand
        const RunArgs a{x.weights, x.biases, x.states, x.points, x.num_points, x.arc_tm, x.arc_tm_shapes,
                        x.num_arc_tm, x.w_extra, x.b_extra, x.iso, x.flip_insideout, nullptr};
        const int rc = guarded(e, [&] {
            run_begin(e, a);
            if (e->run.head < e->run.tail) {
                run_graph_launch(e, kMaxWaves);
                active[(size_t)i] = 1;
            }
        });
        e->lean = false;
        if (rc != AM_OK) return rc;
    }
    int n_active = 0;
    for (char a : active) n_active += a;
    // serve whichever loop has stopped: finished, or waiting for a larger store
    while (n_active > 0) {
        bool progressed = false;
        for (int i = 0; i < count; ++i) {
            if (!active[(size_t)i]) continue;
            am_engine *e = engines[i];
            const cudaError_t q = cudaStreamQuery(e->st);
            if (q == cudaErrorNotReady) continue;
            progressed = true;
            const int rc = guarded(e, [&] {
                AM_CUDA(q);
                if (run_graph_done(e)) {
                    run_graph_launch(e, kMaxWaves);
                } else {
                    active[(size_t)i] = 0;
                    --n_active;
                }
            });
            if (rc != AM_OK) return rc;
        }
        if (!progressed) std::this_thread::yield();
    }
    float wall = 0.f;
    for (int i = 0; i < count; ++i) {
        am_engine *e = engines[i];
        const int rc = guarded(e, [&] {
            run_end(e);
            float ms = 0.f;
            AM_CUDA(cudaEventElapsedTime(&ms, engines[0]->ev0, e->ev1));
            wall = std::max(wall, ms);
        });
        if (rc != AM_OK) return rc;
    }
    if (wall_ms) *wall_ms = wall;
    return AM_OK;
}

// FP64 view of the engine's network for the error report: the engine's own
// parameter copies, converted exactly to double (FP32 engines), same layouts
static NetDev network_fp64(am_engine *e)
{
    if (e->prec == kFloat64) return e->net;
    cudaStream_t st = e->st;
    NetDev n = e->net;
    auto conv = [&](DevBuf &dst, const void *src, long long count) -> const void * {
        if (!src || count <= 0) return src;
        AM_CUDA(dst.reserve(sizeof(double) * (size_t)count));
        launch_to_double(src, count, dst.p, st);
        return dst.p;
    };
    n.W0 = conv(e->w0_64, e->net.W0, 3ll * e->nodes[1]);
    for (int i = 0; i < e->n_lin; ++i) n.bias[i] = conv(e->bias64[i], e->net.bias[i], e->nodes[i + 1]);
    for (int i = 1; i < e->n_lin; ++i) n.Wt[i] = conv(e->wt64[i], e->net.Wt[i], (long long)e->nodes[i] * e->net.Mp[i]);
    int t = 0;
    for (int i = 1; i < e->n_lin; ++i)
        for (int c = 0; c < e->net.nskip[i]; ++c)
            if (e->net.skip[i][c].kind == 1) {
                n.skip[i][c].tmt = conv(e->tmt64[t], e->net.skip[i][c].tmt, e->tm_count[t]);
                ++t;
            }
    if (e->E) {
        n.w_extra = conv(e->wext64, e->net.w_extra, 3ll * e->E);
        n.b_extra = conv(e->bext64, e->net.b_extra, e->E);
    }
    AM_CUDA(cudaGetLastError());
    return n;
}

int am_error_report(am_engine *e, int64_t sample_regions, am_error_report_t *out)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_am) return AM_ERR_NO_RESULT;
    if (!out || sample_regions < 0) return AM_ERR_INVALID_ARGUMENT;
    return guarded(e, [&] {
        cudaStream_t st = e->st;
        const long long R = e->num_regions;
        const long long k = (sample_regions == 0 || sample_regions > R) ? R : sample_regions;
        *out = am_error_report_t{};
        if (k <= 0) return;
        // evenly spaced region ids
        std::vector<long long> ids((size_t)k);
        for (long long j = 0; j < k; ++j) ids[(size_t)j] = (long long)((double)j * (double)R / (double)k);
        for (long long j = 1; j < k; ++j) ids[(size_t)j] = std::max(ids[(size_t)j], ids[(size_t)j - 1] + 1);
        for (long long j = k - 1; j >= 0 && ids[(size_t)j] >= R; --j) ids[(size_t)j] = R - 1 - (k - 1 - j);
        AM_CUDA(e->v_ids.reserve(sizeof(long long) * (size_t)k));
        AM_CUDA(cudaMemcpyAsync(e->v_ids.p, ids.data(), sizeof(long long) * (size_t)k, cudaMemcpyHostToDevice, st));
        const NetDev n64 = network_fp64(e);
        // FP64 rows in slices of at most 1 GiB
        const long long per = (long long)e->ALLP * 4 * (long long)sizeof(double);
        const int slice = (int)std::max<long long>(1, std::min<long long>(k, ((long long)1 << 30) / per));
        AM_CUDA(e->v_keys.reserve(sizeof(uint32_t) * (size_t)slice * e->W));
        AM_CUDA(e->v_rows.reserve((size_t)per * slice));
        AM_CUDA(e->v_eq.reserve(sizeof(double) * 4 * (size_t)slice));
        AM_CUDA(e->v_out.reserve(sizeof(unsigned long long) * 5));
        AM_CUDA(cudaMemsetAsync(e->v_out.p, 0, sizeof(unsigned long long) * 5, st));
        const RegionsDev reg = e->regions();
        for (long long off = 0; off < k; off += slice) {
            const int cnt = (int)std::min<long long>(slice, k - off);
            const long long *dids = e->v_ids.as<long long>() + off;
            launch_gather_keys(e->keys.as<uint32_t>(), e->W, dids, cnt, e->v_keys.as<uint32_t>(), st);
            RegionsDev rr{};
            rr.keys = e->v_keys.as<uint32_t>();
            rr.cap = cnt;
            ChunkDev ch;
            ch.head = 0;
            ch.count = cnt;
            ch.cons = e->v_rows.p;
            ch.eq = e->v_eq.p;
            ch.rec = nullptr;
            launch_compose(kFloat64, n64, rr, ch, e->iso, st);
            launch_verify((int)e->ts, reg, dids, cnt, e->v_rows.as<double>(), e->v_eq.as<double>(), e->ALLP, e->ALL,
                          e->v_out.as<unsigned long long>(), st);
            AM_CUDA(cudaGetLastError());
        }
        unsigned long long h[5];
        AM_CUDA(cudaMemcpyAsync(h, e->v_out.p, sizeof(h), cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        double f, v;
        memcpy(&f, &h[0], sizeof(double));
        memcpy(&v, &h[1], sizeof(double));
        out->faces = (int64_t)h[4];
        out->vertices = (int64_t)h[2];
        out->vertices_singular = (int64_t)h[3];
        out->max_abs_f = f;
        out->max_vertex_err = v;
        e->stats.max_abs_f = f;
        e->stats.max_vertex_err = v;
        e->stats.error_faces = (int64_t)h[4];
    });
}

int am_get_stats(const am_engine *e, am_stats *out)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!out) return AM_ERR_INVALID_ARGUMENT;
    *out = e->stats;
    return AM_OK;
}

// the welded mesh from its device buffers into the engine's host vectors
static void fetch_mesh(am_engine *e)
{
    if (e->mesh_host) return;
    cudaStream_t st = e->st;
    const long long V = e->stats.mesh_num_verts, F = e->stats.mesh_num_faces, I = e->stats.mesh_num_indices;
    e->mesh_verts.resize((size_t)V * 3);
    e->mesh_fs.resize((size_t)F);
    e->mesh_fi.resize((size_t)I);
    if (e->ts == 8) {
        AM_CUDA(cudaMemcpyAsync(e->mesh_verts.data(), e->w_verts.p, sizeof(double) * 3 * V, cudaMemcpyDeviceToHost, st));
    } else {
        std::vector<float> tmp((size_t)V * 3);
        AM_CUDA(cudaMemcpyAsync(tmp.data(), e->w_verts.p, sizeof(float) * 3 * V, cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        for (size_t q = 0; q < tmp.size(); ++q) e->mesh_verts[q] = tmp[q];
    }
    AM_CUDA(cudaMemcpyAsync(e->mesh_fs.data(), e->w_fs.p, sizeof(int) * F, cudaMemcpyDeviceToHost, st));
    AM_CUDA(cudaMemcpyAsync(e->mesh_fi.data(), e->w_fi.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
    AM_CUDA(cudaStreamSynchronize(st));
    e->mesh_host = true;
}

int am_combine_mesh(am_engine *e, double scale, const double *center3)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_am) return AM_ERR_NO_RESULT;
    return guarded(e, [&] {
        cudaStream_t st = e->st;
        const long long R = e->num_regions;
        const long long nr = std::max<long long>(R, 1);
        // the vertex slots in use, compacted (a face has ~4 of its 32)
        AM_CUDA(e->w_voff.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_fflag.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_bsum.reserve(sizeof(int) * (nr / 1024 + 2)));
        AM_CUDA(e->w_counts.reserve(sizeof(long long) * 3));
        WeldBuffers wb{};
        wb.voff = e->w_voff.as<int>();
        wb.fflag = e->w_fflag.as<int>();
        wb.bsum = e->w_bsum.as<int>();
        wb.counts = e->w_counts.as<long long>();
        launch_weld_slots(e->regions(), R, wb, st);
        AM_CUDA(cudaGetLastError());
        long long V = 0;
        AM_CUDA(cudaMemcpyAsync(&V, wb.counts, sizeof(long long), cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        AM_CHECK(V < (1ll << 30), "too many polygon vertices for one mesh (2^30)");
        const long long ns = std::max<long long>(V, 1);
        unsigned long long tcap = 1;
        while (tcap < (unsigned long long)ns * 2ull) tcap <<= 1;
        AM_CUDA(e->w_vsid.reserve(sizeof(long long) * ns));
        AM_CUDA(e->w_table.reserve(sizeof(unsigned long long) * tcap));
        AM_CUDA(e->w_rep.reserve(sizeof(int) * ns));
        AM_CUDA(e->w_wslot.reserve(sizeof(unsigned) * ns));
        AM_CUDA(e->w_flag.reserve(sizeof(int) * ns));
        AM_CUDA(e->w_vidx.reserve(sizeof(int) * ns));
        AM_CUDA(e->w_bsum.reserve(sizeof(int) * (std::max(ns, nr) / 1024 + 2)));
        AM_CUDA(e->w_fsize.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_fid.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_foff.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_verts.reserve(e->ts * 3 * ns));
        AM_CUDA(e->w_fs.reserve(sizeof(int) * (nr + 1)));
        AM_CUDA(e->w_fi.reserve(sizeof(int) * ns));
        wb.vsid = e->w_vsid.as<long long>();
        wb.table = e->w_table.as<unsigned long long>();
        wb.mask = tcap - 1;
        wb.rep = e->w_rep.as<int>();
        wb.wslot = e->w_wslot.as<unsigned>();
        wb.flag = e->w_flag.as<int>();
        wb.vidx = e->w_vidx.as<int>();
        wb.bsum = e->w_bsum.as<int>();
        wb.fsize = e->w_fsize.as<int>();
        wb.fid = e->w_fid.as<int>();
        wb.foff = e->w_foff.as<int>();
        wb.out_verts = e->w_verts.p;
        wb.face_sizes = e->w_fs.as<int>();
        wb.face_idx = e->w_fi.as<int>();
        const double c0[3] = {0, 0, 0};
        AM_CUDA(cudaMemsetAsync(e->d_err.p, 0, sizeof(int), st));
        launch_weld(e->prec, e->weld_mode, e->N, e->W, e->regions(), R, V, wb, scale, center3 ? center3 : c0, e->flip,
                    e->d_err.as<int>(), st);
        AM_CUDA(cudaGetLastError());
        long long cnt[3] = {0, 0, 0};
        AM_CUDA(cudaMemcpyAsync(cnt, wb.counts, sizeof(cnt), cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        e->check_err();
        e->stats.mesh_num_verts = cnt[0];
        e->stats.mesh_num_faces = cnt[1];
        e->stats.mesh_num_indices = cnt[2];
        e->has_mesh = true;
        e->mesh_host = false; // read back on demand: am_get_mesh copies straight into the caller's arrays
        // large weld buffers go back (many engines of a batch weld one after
        // the other): their mesh moves to the host first
        DevBuf *weld[] = {&e->w_table, &e->w_rep, &e->w_flag, &e->w_vidx, &e->w_bsum, &e->w_fflag, &e->w_fsize,
                          &e->w_fid, &e->w_foff, &e->w_verts, &e->w_fs, &e->w_fi, &e->w_voff, &e->w_vsid,
                          &e->w_wslot};
        size_t held = 0;
        for (DevBuf *b : weld) held += b->bytes;
        if (held > ((size_t)8 << 30)) {
            fetch_mesh(e);
            for (DevBuf *b : weld) b->reset();
        }
    });
}

int am_get_mesh(am_engine *e, double *verts, int32_t *face_sizes, int32_t *face_indices)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_mesh) return AM_ERR_NO_RESULT;
    if (e->mesh_host) {
        if (verts) std::copy(e->mesh_verts.begin(), e->mesh_verts.end(), verts);
        if (face_sizes) std::copy(e->mesh_fs.begin(), e->mesh_fs.end(), face_sizes);
        if (face_indices) std::copy(e->mesh_fi.begin(), e->mesh_fi.end(), face_indices);
        return AM_OK;
    }
    return guarded(e, [&] { // from the weld buffers straight into the caller's arrays
        cudaStream_t st = e->st;
        const long long V = e->stats.mesh_num_verts, F = e->stats.mesh_num_faces, I = e->stats.mesh_num_indices;
        std::vector<float> tmp;
        if (verts && V > 0) {
            if (e->ts == 8) {
                AM_CUDA(cudaMemcpyAsync(verts, e->w_verts.p, sizeof(double) * 3 * V, cudaMemcpyDeviceToHost, st));
            } else {
                tmp.resize((size_t)V * 3);
                AM_CUDA(cudaMemcpyAsync(tmp.data(), e->w_verts.p, sizeof(float) * 3 * V, cudaMemcpyDeviceToHost, st));
            }
        }
        if (face_sizes && F > 0)
            AM_CUDA(cudaMemcpyAsync(face_sizes, e->w_fs.p, sizeof(int) * F, cudaMemcpyDeviceToHost, st));
        if (face_indices && I > 0)
            AM_CUDA(cudaMemcpyAsync(face_indices, e->w_fi.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        for (size_t q = 0; q < tmp.size(); ++q) verts[q] = tmp[q];
    });
}

int am_export_mesh(am_engine *e, const char *file_path, int is_polymesh, int is_float32)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_mesh) return AM_ERR_NO_RESULT;
    if (!file_path) return AM_ERR_INVALID_ARGUMENT;
    if (!e->mesh_host) {
        const int rc = guarded(e, [&] { fetch_mesh(e); });
        if (rc != AM_OK) return rc;
    }
    FILE *f = fopen(file_path, "wb");
    if (!f) {
        e->last_error = std::string("cannot open ") + file_path;
        return AM_ERR_IO;
    }
    const long long V = e->stats.mesh_num_verts, F = e->stats.mesh_num_faces;
    long long tri = 0;
    if (!is_polymesh)
        for (long long i = 0; i < F; ++i) tri += e->mesh_fs[i] - 2;
    // header as polymesh.h:368-377
    fprintf(f, "ply\nformat binary_little_endian 1.0\nelement vertex %lld\n", V);
    const char *ty = is_float32 ? "float" : "double";
    fprintf(f, "property %s x\nproperty %s y\nproperty %s z\n", ty, ty, ty);
    fprintf(f, "element face %lld\nproperty list uchar int vertex_index\nend_header\n", is_polymesh ? F : tri);
    bool ok = true;
    for (long long i = 0; i < V && ok; ++i) {
        if (is_float32) {
            const float v[3] = {(float)e->mesh_verts[3 * i], (float)e->mesh_verts[3 * i + 1], (float)e->mesh_verts[3 * i + 2]};
            ok = fwrite(v, sizeof(float), 3, f) == 3;
        } else {
            ok = fwrite(&e->mesh_verts[3 * i], sizeof(double), 3, f) == 3;
        }
    }
    size_t off = 0;
    for (long long i = 0; i < F && ok; ++i) {
        const int n = e->mesh_fs[i];
        const int32_t *idx = e->mesh_fi.data() + off;
        if (is_polymesh) {
            const unsigned char c = (unsigned char)n;
            ok = fwrite(&c, 1, 1, f) == 1 && fwrite(idx, sizeof(int32_t), n, f) == (size_t)n;
        } else {
            const unsigned char c = 3;
            for (int j = 0; j + 2 < n && ok; ++j) {
                const int32_t t[3] = {idx[0], idx[j + 1], idx[j + 2]};
                ok = fwrite(&c, 1, 1, f) == 1 && fwrite(t, sizeof(int32_t), 3, f) == 3;
            }
        }
        off += n;
    }
    if (fclose(f) != 0) ok = false;
    if (!ok) {
        e->last_error = std::string("write failed: ") + file_path;
        return AM_ERR_IO;
    }
    return AM_OK;
}

int am_get_regions(am_engine *e, uint32_t *bits, int32_t *nverts, double *verts, int32_t *edges, int8_t *status,
                   double *seeds, int32_t *start)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_am) return AM_ERR_NO_RESULT;
    return guarded(e, [&] {
        cudaStream_t st = e->st;
        const long long R = e->num_regions;
        if (bits) AM_CUDA(cudaMemcpyAsync(bits, e->keys.p, sizeof(uint32_t) * e->W * R, cudaMemcpyDeviceToHost, st));
        if (nverts) AM_CUDA(cudaMemcpyAsync(nverts, e->nv.p, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, st));
        if (edges) AM_CUDA(cudaMemcpyAsync(edges, e->edges.p, sizeof(int32_t) * kVMax * R, cudaMemcpyDeviceToHost, st));
        if (status) AM_CUDA(cudaMemcpyAsync(status, e->status.p, R, cudaMemcpyDeviceToHost, st));
        if (start) AM_CUDA(cudaMemcpyAsync(start, e->start.p, sizeof(int32_t) * R, cudaMemcpyDeviceToHost, st));
        if (verts || seeds) {
            std::vector<unsigned char> vb(verts ? e->ts * 3 * kVMax * R : 0), mb(seeds ? e->ts * 4 * R : 0);
            if (verts) AM_CUDA(cudaMemcpyAsync(vb.data(), e->verts.p, vb.size(), cudaMemcpyDeviceToHost, st));
            if (seeds) AM_CUDA(cudaMemcpyAsync(mb.data(), e->mid.p, mb.size(), cudaMemcpyDeviceToHost, st));
            AM_CUDA(cudaStreamSynchronize(st));
            const size_t nvv = (size_t)3 * kVMax * R;
            if (verts)
                for (size_t q = 0; q < nvv; ++q)
                    verts[q] = e->ts == 8 ? ((const double *)vb.data())[q] : (double)((const float *)vb.data())[q];
            if (seeds)
                for (long long r = 0; r < R; ++r)
                    for (int c = 0; c < 3; ++c)
                        seeds[3 * r + c] = e->ts == 8 ? ((const double *)mb.data())[4 * r + c]
                                                      : (double)((const float *)mb.data())[4 * r + c];
        }
        AM_CUDA(cudaStreamSynchronize(st));
    });
}

int am_region_rows(am_engine *e, int64_t first, int count, double *rows, double *eq)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (!e->has_am) return AM_ERR_NO_RESULT;
    if (first < 0 || count < 0 || first + count > e->num_regions) return AM_ERR_INVALID_ARGUMENT;
    return guarded(e, [&] {
        cudaStream_t st = e->st;
        if (count == 0) return;
        e->ensure_chunk(count);
        ChunkDev ch;
        ch.head = first;
        ch.count = count;
        ch.cons = e->cons.p;
        ch.eq = e->eq.p;
        ch.rec = e->rec.as<int32_t>();
        AM_CUDA(cudaMemsetAsync(e->d_err.p, 0, sizeof(int), st));
        if (e->prec == kMixed)
            launch_compose_tc(e->net, e->tcnet, e->regions(), ch, e->iso, e->d_err.as<int>(), st);
        else
            launch_compose(e->prec, e->net, e->regions(), ch, e->iso, st);
        AM_CUDA(cudaGetLastError());
        const size_t nrow = (size_t)count * e->ALLP * 4;
        std::vector<unsigned char> rb(nrow * e->tc), eb((size_t)count * 4 * e->tc);
        AM_CUDA(cudaMemcpyAsync(rb.data(), e->cons.p, rb.size(), cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaMemcpyAsync(eb.data(), e->eq.p, eb.size(), cudaMemcpyDeviceToHost, st));
        AM_CUDA(cudaStreamSynchronize(st));
        e->check_err();
        auto get = [&](const std::vector<unsigned char> &b, size_t q) {
            return e->tc == 8 ? ((const double *)b.data())[q] : (double)((const float *)b.data())[q];
        };
        for (int r = 0; r < count; ++r)
            for (int k = 0; k < e->ALL; ++k)
                for (int c = 0; c < 4; ++c)
                    if (rows) rows[((size_t)r * e->ALL + k) * 4 + c] = get(rb, ((size_t)r * e->ALLP + k) * 4 + c);
        if (eq)
            for (size_t q = 0; q < (size_t)count * 4; ++q) eq[q] = get(eb, q);
    });
}

int am_destroy(am_engine *e)
{
    if (!e) return AM_ERR_NOT_INITIALIZED;
    if (e->st) cudaStreamSynchronize(e->st);
    delete e;
    return AM_OK;
}

} // extern "C"
