// am_polygon.cu -- face polygon of every region of a chunk, warp per face,
// plus the frontier insert of its neighbours.
//
// The face of a region is the polygon {x : w_eq.x + b_eq = 0, C_k(x) <= 0 for
// all k}.  The reference finds it by a pivot walk that tries candidate planes
// in order of distance from a seed point, one 3x3 solve plus an N-row
// feasibility scan per candidate, one candidate per region per round with a
// host round trip between rounds (backend/inc/kernel.h:1258-1320).  Here one
// warp owns a face: the region's constraint rows are staged in shared memory
// and the walk is ray shooting along the current edge line -- a single pass
// over the rows gives the first plane the line hits, and the vertex is the
// 3x3 solve of (edge plane, hit plane, face plane).  The walk goes
// counter-clockwise about w_eq, which is the orientation the reference's
// correctNormalDirection enforces (kernel.h:1325-1370).  Zero-length edges
// (vertices closer than FP_SAME_EPS in L1) are merged and spawn no neighbour,
// as in cudaUpdateVert_kernel (kernel.h:1197-1205).
//
// Seed regions (start == -1) first find a polygon vertex exactly as the
// reference's calcStartIdx does (kernel.h:799-856): planes ordered by signed
// geometric distance from the seed point, pairs enumerated by get_i_j up to
// x = min((ALL-1)(ALL-2), 812), the first pair whose vertex satisfies every
// other constraint within FP_EPS wins.  Those pairs only involve the 57
// nearest planes, so a partial selection replaces the reference's full sort.
//
// Every edge on a hidden unit's plane gives a neighbour: the key with that
// bit flipped.  Its hash is updated in O(1) and it is inserted into the
// region hash set (full-key comparison on fingerprint match); among equal new
// keys the smallest (parent, plane) id wins, so the result is deterministic.
#include <cuda/atomic>
#include <cuda_runtime.h>

#include "am_device.cuh"
#include "am_internal.h"
#include "am_umma.cuh"

namespace am {

namespace {

template <typename T>
__device__ __forceinline__ unsigned long long order_key(T d);
template <>
__device__ __forceinline__ unsigned long long order_key<float>(float d)
{
    if (d != d) return 0ull;
    uint32_t u = __float_as_uint(d);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return (unsigned long long)u;
}
template <>
__device__ __forceinline__ unsigned long long order_key<double>(double d)
{
    if (d != d) return 0ull;
    unsigned long long u = (unsigned long long)__double_as_longlong(d);
    u = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    return u;
}

// (key, index) pairs: a is ahead of b when its distance is larger, ties by lower index
__device__ __forceinline__ bool ahead(unsigned long long ka, int ia, unsigned long long kb, int ib)
{
    return ka > kb || (ka == kb && ia < ib);
}

__device__ __forceinline__ bool finite_bits(float v) { return (__float_as_uint(v) & 0x7f800000u) != 0x7f800000u; }
__device__ __forceinline__ bool finite_bits(double v)
{
    return ((uint32_t)(__double_as_longlong(v) >> 52) & 0x7ffu) != 0x7ffu;
}

// The vertex of planes a, b and the face plane, solved by the warp: lanes
// 0-7 convert the two rows' components (one conversion instruction), lane
// L = 0..3 (and its copies L + 4, L + 8, ...) computes Cramer's determinant
// with column L - 1 replaced by -b (L = 0: none), then divides by the lane-0
// determinant -- the same arithmetic as solve3 on one lane, in three
// dependent FP64 sequences (convert, determinant, divide) instead of forty,
// which matters because the SM's FP64 pipe issues a warp instruction at the
// same cost however few lanes are active.  Every lane returns the vertex in
// the solve precision (V) and rounded to the scan precision (Vc); false if a
// coordinate is not finite.
template <typename TC, typename TS>
__device__ __forceinline__ bool warp_solve(const vec4_t<TC> *rows, int a, int b, const TS *eqv, TS *V, TC *Vc,
                                           int lane)
{
    const TC *ra = reinterpret_cast<const TC *>(rows + a);
    const TC *rb = reinterpret_cast<const TC *>(rows + b);
    const int c = lane & 7;
    const TS cs = (TS)(c < 4 ? ra[c] : rb[c - 4]);
    TS m[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) m[j] = __shfl_sync(0xffffffffu, cs, j);
    const int L = lane & 3;
    const TS a00 = L == 1 ? -m[3] : m[0], a01 = L == 2 ? -m[3] : m[1], a02 = L == 3 ? -m[3] : m[2];
    const TS a10 = L == 1 ? -m[7] : m[4], a11 = L == 2 ? -m[7] : m[5], a12 = L == 3 ? -m[7] : m[6];
    const TS a20 = L == 1 ? -eqv[3] : eqv[0], a21 = L == 2 ? -eqv[3] : eqv[1], a22 = L == 3 ? -eqv[3] : eqv[2];
    const TS d = det3<TS>(a00, a01, a02, a10, a11, a12, a20, a21, a22);
    const TS d0 = __shfl_sync(0xffffffffu, d, 0);
    const TS x = d / d0;
    const TC xc = (TC)x;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        V[j] = __shfl_sync(0xffffffffu, x, j + 1);
        Vc[j] = __shfl_sync(0xffffffffu, xc, j + 1);
    }
    return finite_bits(V[0]) && finite_bits(V[1]) && finite_bits(V[2]);
}

// L1 distance test |V - P|_1 < eps.  With TS wider than TC it is decided on
// the scan-precision copies when the rounding margin allows -- Vc and Pc are
// V and P rounded to nearest, so the TC sum is within 2^-23 (|Vc|_1 + |Pc|_1)
// + 3 ulp of the exact one; 2^-21 (|Vc|_1 + |Pc|_1 + d) bounds both -- and
// returns -1 ("near") otherwise, for the caller to decide in TS.
template <typename TC, typename TS>
__device__ __forceinline__ int same_filter(const TC *Vc, TC px, TC py, TC pz, TS eps)
{
    const TC d = fabs(Vc[0] - px) + fabs(Vc[1] - py) + fabs(Vc[2] - pz);
    const TC mag = fabs(Vc[0]) + fabs(Vc[1]) + fabs(Vc[2]) + fabs(px) + fabs(py) + fabs(pz);
    const TC margin = TC(4.76837158203125e-7) * (mag + d); // 2^-21
    const TC e = (TC)eps;
    if (d >= e + margin) return 0;
    if (d + margin < e) return 1;
    return -1;
}

__device__ __forceinline__ long long next_work(WaveCtl *ctl, int lane)
{
    unsigned int v = 0;
    if (lane == 0) v = atomicAdd(&ctl->work, 1u);
    return (long long)__shfl_sync(0xffffffffu, v, 0);
}

__device__ __forceinline__ unsigned long long load_slot(const unsigned long long *p)
{
    cuda::atomic_ref<unsigned long long, cuda::thread_scope_device> a(*const_cast<unsigned long long *>(p));
    return a.load(cuda::memory_order_relaxed);
}

// Does the key stored behind slot value `cur` equal parent_key ^ flip(k)?
// Region entries (tag 0) point at the region store; candidate entries (tag 1)
// carry (chunk-local parent, plane) and point at the parent's key.  The whole
// warp compares: lane l takes words l, l + 32, ..., all loads issued at once.
__device__ bool warp_key_matches(unsigned long long cur, const RegionsDev &reg, long long head, int ALL, int W,
                                 const uint32_t *pkey, int k, int lane)
{
    const uint32_t id = (uint32_t)cur & 0x7fffffffu;
    const bool cand = (cur >> 31) & 1ull;
    const uint32_t *other;
    int ok2 = -1;
    if (cand) {
        other = reg.keys + (size_t)(head + id / ALL) * W;
        ok2 = (int)(id % ALL);
    } else {
        other = reg.keys + (size_t)id * W;
    }
    const int kw = k >> 5;
    const uint32_t kb = 1u << (k & 31);
    const int ow = ok2 >= 0 ? (ok2 >> 5) : -1;
    const uint32_t ob = ok2 >= 0 ? (1u << (ok2 & 31)) : 0u;
    bool differ = false;
    for (int w = lane; w < W; w += 32) {
        const uint32_t a = pkey[w] ^ (w == kw ? kb : 0u);
        const uint32_t b = other[w] ^ (w == ow ? ob : 0u);
        differ = differ || a != b;
    }
    return !__any_sync(0xffffffffu, differ);
}

// Insert the neighbour across plane k (parent key pkey with bit k flipped)
// into the region hash set; the whole warp works on it, lane 0 owning the
// slot operations.  Returns the slot claimed for a new candidate (or the
// candidate slot this one now shares), -1 when the key is a committed
// region already.  Among equal candidate keys the smallest (parent, plane)
// id stays in the slot, so the result does not depend on timing.
__device__ int warp_insert(const RegionsDev &reg, const HashDev &hs, long long head, int ALL, int W, const uint32_t *pkey,
                           uint64_t phash, long long rl, int k, int lane, int *err)
{
    const unsigned full = 0xffffffffu;
    const uint64_t h = flip_hash(phash, pkey[k >> 5], k);
    const uint32_t fp = fp_of(h);
    const uint32_t myid = (uint32_t)(rl * ALL + k);
    const unsigned long long mine = slot_value(fp, 1, myid);
    unsigned long long slot = h & hs.mask;
    for (int probe = 0; probe < kMaxProbes; ++probe) {
        unsigned long long cur = 0ull;
        int claimed = 0;
        if (lane == 0) {
            cur = load_slot(hs.slots + slot);
            if (cur == kEmpty) {
                const unsigned long long old = atomicCAS(hs.slots + slot, kEmpty, mine);
                claimed = old == kEmpty;
                cur = old;
            }
        }
        cur = __shfl_sync(full, cur, 0);
        if (__shfl_sync(full, claimed, 0)) return (int)slot;
        if ((uint32_t)(cur >> 32) == fp && warp_key_matches(cur, reg, head, ALL, W, pkey, k, lane)) {
            if ((cur >> 31) & 1ull) {
                if (lane == 0) atomicMin(hs.slots + slot, mine);
                return (int)slot;
            }
            return -1;
        }
        slot = (slot + (unsigned long long)probe + 1ull) & hs.mask;
    }
    if (lane == 0) atomicOr(err, kErrTableFull);
    return -1;
}

// A face belongs to a group of G warps (G = 1, 2, 4 or 8; wide networks use
// more, so that a block holds fewer faces' rows and more warps).  The group
// stages the rows together, and every warp of it runs the same walk on them:
// each scans rows k = 32 gw + lane (mod 32 G), the partial (t, plane) minima
// meet in shared memory (two slots, by step parity) behind one named barrier
// per step, and every warp takes the same minimum, so the group stays in
// step without further messages.  Warp 0 (the leader) alone re-solves the
// vertices in the solve precision and writes the outputs.  G = 1 is the plain
// warp per face with no barrier.
constexpr int kListCap = 384;  // rows the pruned walk keeps at most (more: the walk scans every row)
constexpr int kPruneMin = 96;  // fewer rows than this: no pruning
constexpr int kRowWaitIters = 1 << 22; // bound of the wait for a face's rows (bulk copy)

template <typename TC>
struct GroupShared {
    long long rl;   // the group's region (chunk-local)
    uint64_t rbar;  // the face's rows have landed (bulk copy)
    int done, near; // the leader's refinement outcome; a warp met a row near a vertex
    TC bt[2][8];    // partial minima per step parity and warp
    double btd[2][8]; // the same for a scan in FP64 over FP32 rows
    int bk[2][8];
    int nlist;      // rows kept by the pruning
    // phases of a face, one at a time (a barrier between any two): the seed
    // start search; row pruning, first the sample's extreme rows per warp
    // and direction, then (once every warp has read those) the list of the
    // rows kept, read by the walk; the neighbour planes by edge after it
    union {
        struct {
            unsigned long long sk[2][8]; // partial choices of a selection pass
            double sv[3];                // the start vertex found ...
            int sri;                     // ... and its plane
        } seed;
        struct {
            TC v[8][8];
            int16_t i[8][8];
        } ext;
        uint16_t list[kListCap];
        int ve[kVMax]; // -1: no neighbour across the edge (from the leader)
    };
};

template <typename TC>
struct Grp {
    int G, gw, bar;
    GroupShared<TC> *sh;
    // named barrier 1 + group (at most four groups per block when G > 1);
    // constant ids, so that a block reserves five barriers, not sixteen
    __device__ __forceinline__ void sync() const
    {
        const int n = 32 * G;
        switch (bar) {
        case 1: asm volatile("bar.sync 1, %0;" ::"r"(n) : "memory"); break;
        case 2: asm volatile("bar.sync 2, %0;" ::"r"(n) : "memory"); break;
        case 3: asm volatile("bar.sync 3, %0;" ::"r"(n) : "memory"); break;
        default: asm volatile("bar.sync 4, %0;" ::"r"(n) : "memory"); break;
        }
    }
};

template <typename TC>
__host__ __device__ constexpr size_t group_shared_bytes()
{
    return (sizeof(GroupShared<TC>) + 15) / 16 * 16;
}

// first hit along the edge line over rows k0, k0 + kstep, ... (of the kept
// list, when the rows were pruned): min over crossing planes of
// t = max(0, -g) / a, compared as fractions within a lane (two interleaved
// candidates per lane halve the compare chain), then across the warp; every
// lane returns the warp's (t, plane), plane 0x7fffffff if none.  The rows are
// TR, the arithmetic TA (FP64 over FP32 rows for the mixed form's FP64
// predicates).  kNear: `near` is set when a row other than the two the
// current point lies on has |g| < 1e-6 there (the rows are normalised, so g
// is a distance): a predicate near zero, which the mixed form takes again in
// FP64.
template <typename TR, typename TA, bool kNear>
__device__ __forceinline__ void hit_scan(const vec4_t<TR> *rows, int ALL, const uint16_t *list, int nlist, int k0,
                                         int kstep, TA d0, TA d1, TA d2, TA thr, TA c0, TA c1, TA c2, int e, int prev,
                                         TA &bt_out, int &bk_out, bool &near)
{
    TA bnum = TA(1), bden = TA(0), bnum1 = TA(1), bden1 = TA(0);
    int bk = 0x7fffffff, bk1 = 0x7fffffff;
    bool nr = false;
    // rows of one chain come in increasing k, so that a later row never
    // wins a tie against the chain's earlier choice: the index test is only
    // needed for the pruning list, whose rows come in any order
    auto consider = [&](int k, TA &bn, TA &bd, int &bi, bool any_order) {
        const vec4_t<TR> r = rows[k];
        const TA rx = (TA)r.x, ry = (TA)r.y, rz = (TA)r.z, rw = (TA)r.w;
        const TA a = rx * d0 + ry * d1 + rz * d2;
        TA num;
        if (kNear) {
            num = -(rx * c0 + ry * c1 + rz * c2 + rw);
            nr = nr || (fabs(num) < TA(1e-6) && k != e && k != prev);
            if (!(a > thr) || k == e || k == prev) return;
        } else {
            if (!(a > thr) || k == e || k == prev) return;
            num = -(rx * c0 + ry * c1 + rz * c2 + rw);
        }
        num = num > TA(0) ? num : TA(0);
        const TA lhs = num * bd, rhs = bn * a;
        if (lhs < rhs || (any_order && lhs == rhs && k < bi)) {
            bn = num;
            bd = a;
            bi = k;
        }
    };
    if (list) { // the rows that survived pruning
        int j = k0;
        for (; j + kstep < nlist; j += 2 * kstep) {
            consider(list[j], bnum, bden, bk, true);
            consider(list[j + kstep], bnum1, bden1, bk1, true);
        }
        if (j < nlist) consider(list[j], bnum, bden, bk, true);
    } else {
        int k = k0;
#pragma unroll 2
        for (; k + kstep < ALL; k += 2 * kstep) {
            consider(k, bnum, bden, bk, false);
            consider(k + kstep, bnum1, bden1, bk1, false);
        }
        if (k < ALL) consider(k, bnum, bden, bk, false);
    }
    {
        const TA lhs = bnum1 * bden, rhs = bnum * bden1;
        if (bk1 != 0x7fffffff && (lhs < rhs || (lhs == rhs && bk1 < bk))) {
            bnum = bnum1;
            bden = bden1;
            bk = bk1;
        }
    }
    TA bt = bk == 0x7fffffff ? TA(INFINITY) : bnum / bden;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const TA ot = __shfl_xor_sync(0xffffffffu, bt, o);
        const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (ot < bt || (ot == bt && ok < bk)) {
            bt = ot;
            bk = ok;
        }
    }
    bt_out = bt;
    bk_out = bk;
    if (kNear) near = __any_sync(0xffffffffu, nr);
}

// The mixed form's scan with FP64 predicates (over FP32 rows): every row is
// evaluated in FP32 from the FP32 copy of the current point, and again in
// FP64 from the FP64 current point when that value is within 2e-6 of zero --
// a sign or feasibility decision near zero, taken in FP64.  The first hit is
// the smaller of the FP32 candidates' best and the FP64 candidates' best,
// compared in FP64, ties to the lower row.
__device__ __forceinline__ void hit_scan_wide(const float4 *rows, int ALL, const uint16_t *list, int nlist, int k0,
                                              int kstep, float d0, float d1, float d2, float thr, float c0, float c1,
                                              float c2, double D0, double D1, double D2, double thr64, double C0,
                                              double C1, double C2, int e, int prev, double &bt_out, int &bk_out)
{
    float bnum = 1.f, bden = 0.f;
    int bk = 0x7fffffff;
    double tn = INFINITY;
    int tk = 0x7fffffff;
    auto consider = [&](int k) {
        if (k == e || k == prev) return;
        const float4 r = rows[k];
        const float g = r.x * c0 + r.y * c1 + r.z * c2 + r.w;
        if (fabsf(g) < 2e-6f) {
            const double a = (double)r.x * D0 + (double)r.y * D1 + (double)r.z * D2;
            if (!(a > thr64)) return;
            double num = -((double)r.x * C0 + (double)r.y * C1 + (double)r.z * C2 + (double)r.w);
            num = num > 0.0 ? num : 0.0;
            const double t = num / a;
            if (t < tn || (t == tn && k < tk)) {
                tn = t;
                tk = k;
            }
            return;
        }
        const float a = r.x * d0 + r.y * d1 + r.z * d2;
        if (!(a > thr)) return;
        const float num = -g > 0.f ? -g : 0.f;
        const float lhs = num * bden, rhs = bnum * a;
        if (lhs < rhs || (lhs == rhs && k < bk)) {
            bnum = num;
            bden = a;
            bk = k;
        }
    };
    if (list) {
        for (int j = k0; j < nlist; j += kstep) consider(list[j]);
    } else {
        for (int k = k0; k < ALL; k += kstep) consider(k);
    }
    double bt = bk == 0x7fffffff ? INFINITY : (double)bnum / (double)bden;
    if (tk != 0x7fffffff && (tn < bt || (tn == bt && tk < bk))) {
        bt = tn;
        bk = tk;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double ot = __shfl_xor_sync(0xffffffffu, bt, o);
        const int ok = __shfl_xor_sync(0xffffffffu, bk, o);
        if (ot < bt || (ot == bt && ok < bk)) {
            bt = ot;
            bk = ok;
        }
    }
    bt_out = bt;
    bk_out = bk;
}

// One face walk: from the start plane s, ray shooting along each edge line,
// the scan in TA (TC, or TS for the mixed form's FP64 predicates), vertices
// solved in TS.  Lane i ends with vertex i (vx, vy, vz) and the plane of the
// edge leaving it (ve); lane j records step j's hit plane (sbk) and merge
// decision (sdec, 0 append, 1 merge with the previous vertex, 2 merge with
// the first), nsteps the steps taken.  kNear: `near` (this warp) is set when
// some step's scan met a row within 1e-6 of the current point.
template <typename TC, typename TS, bool kGroup, typename TA = TC, bool kNear = false>
__device__ void walk(const vec4_t<TC> *rows, int ALL, const uint16_t *list, int nlist, const vec4_t<TC> &eqc,
                     const TS *eqv, const TS *p, int s, TC par_eps, TS same_eps, int lane, TS &vx, TS &vy, TS &vz,
                     int &ve, int &n, bool &closed, int8_t &status, int &sbk, int &sdec, int &nsteps, const Grp<TC> &g,
                     bool *near = nullptr)
{
    constexpr bool kWide = sizeof(TA) > sizeof(TC); // FP64 scan over FP32 rows
    TC cx = 0, cy = 0, cz = 0; // the vertex rounded to the scan precision
    vx = vy = vz = TS(0);
    ve = -1;
    n = 0;
    closed = false;
    sbk = -1;
    sdec = 0;
    nsteps = 0;
    int e = s, prev = -1;
    bool any_near = false;
    TC curc[3] = {(TC)p[0], (TC)p[1], (TC)p[2]}; // current point, scan precision
    TA cur[3] = {(TA)p[0], (TA)p[1], (TA)p[2]};  // and in FP64 for the wide scan
    for (int step = 0; step < kWalkSteps; ++step) {
        nsteps = step + 1;
        // direction of the edge line: w_eq x w_e (counter-clockwise about w_eq)
        const vec4_t<TC> ref_ = rows[e];
        const TC d0 = eqc.y * ref_.z - eqc.z * ref_.y;
        const TC d1 = eqc.z * ref_.x - eqc.x * ref_.z;
        const TC d2 = eqc.x * ref_.y - eqc.y * ref_.x;
        const TC thr = par_eps * sqrt(d0 * d0 + d1 * d1 + d2 * d2);
        // first hit along the edge line, the scan split over the group
        TA bt;
        int bk;
        if constexpr (kWide) {
            const TA q0 = (TA)eqv[0], q1 = (TA)eqv[1], q2 = (TA)eqv[2];
            const TA rx = (TA)ref_.x, ry = (TA)ref_.y, rz = (TA)ref_.z;
            const TA D0 = q1 * rz - q2 * ry, D1 = q2 * rx - q0 * rz, D2 = q0 * ry - q1 * rx;
            const TA thr64 = (TA)par_eps * sqrt(D0 * D0 + D1 * D1 + D2 * D2);
            hit_scan_wide(rows, ALL, list, nlist, kGroup ? 32 * g.gw + lane : lane, kGroup ? 32 * g.G : 32, d0, d1, d2,
                          thr, curc[0], curc[1], curc[2], D0, D1, D2, thr64, cur[0], cur[1], cur[2], e, prev, bt, bk);
        } else {
            bool nr = false;
            hit_scan<TC, TC, kNear>(rows, ALL, list, nlist, kGroup ? 32 * g.gw + lane : lane, kGroup ? 32 * g.G : 32, d0,
                                    d1, d2, thr, curc[0], curc[1], curc[2], e, prev, bt, bk, nr);
            any_near = any_near || nr;
        }
        if (kGroup) {
            const int par = step & 1;
            TA *sbt = kWide ? (TA *)&g.sh->btd[par][0] : (TA *)&g.sh->bt[par][0];
            if (lane == 0) {
                sbt[g.gw] = bt;
                g.sh->bk[par][g.gw] = bk;
            }
            g.sync();
            bt = sbt[0];
            bk = g.sh->bk[par][0];
            for (int w = 1; w < g.G; ++w) {
                const TA ot = sbt[w];
                const int ok = g.sh->bk[par][w];
                if (ot < bt || (ot == bt && ok < bk)) {
                    bt = ot;
                    bk = ok;
                }
            }
        }
        if (bk == 0x7fffffff) { // the edge line never leaves the region
            status = kOpen;
            break;
        }
        // vertex = 3x3 solve of (edge plane, hit plane, face plane)
        TS V[3];
        TC Vc[3];
        if (!warp_solve<TC, TS>(rows, e, bk, eqv, V, Vc, lane)) {
            status = kSingular;
            break;
        }
        // 0 append, 1 zero-length edge on e (merge), 2 zero-length closing edge;
        // decided in the solve precision (on the scan-precision copies
        // where the rounding margin settles it)
        int decision = 0;
        if (n > 0) {
            int s1 = -1, s2 = 0;
            if (sizeof(TS) > sizeof(TC)) {
                s1 = same_filter<TC, TS>(Vc, __shfl_sync(0xffffffffu, cx, n - 1),
                                         __shfl_sync(0xffffffffu, cy, n - 1),
                                         __shfl_sync(0xffffffffu, cz, n - 1), same_eps);
                if (bk == s && s1 == 0)
                    s2 = same_filter<TC, TS>(Vc, __shfl_sync(0xffffffffu, cx, 0),
                                             __shfl_sync(0xffffffffu, cy, 0),
                                             __shfl_sync(0xffffffffu, cz, 0), same_eps);
            }
            if (s1 == 1) {
                decision = 1;
            } else if (s1 == 0 && s2 != -1) {
                decision = s2 == 1 ? 2 : 0;
            } else {
                const TS lx = __shfl_sync(0xffffffffu, vx, n - 1);
                const TS ly = __shfl_sync(0xffffffffu, vy, n - 1);
                const TS lz = __shfl_sync(0xffffffffu, vz, n - 1);
                if (lane == 0) { // in the solve precision, on one lane
                    if (fabs(V[0] - lx) + fabs(V[1] - ly) + fabs(V[2] - lz) < same_eps)
                        decision = 1;
                    else if (bk == s && fabs(V[0] - vx) + fabs(V[1] - vy) + fabs(V[2] - vz) < same_eps)
                        decision = 2;
                }
                decision = __shfl_sync(0xffffffffu, decision, 0);
            }
        }
        if (lane == step) {
            sbk = bk;
            sdec = decision;
        }
        if (decision == 1 && lane == n - 1) ve = bk; // the edge on e has zero length
        const bool appended = (decision == 0);
        if (appended) {
            if (lane == n) {
                vx = V[0];
                vy = V[1];
                vz = V[2];
                cx = Vc[0];
                cy = Vc[1];
                cz = Vc[2];
                ve = bk;
            }
            n++;
        }
        if (bk == s) {
            closed = true;
            break;
        }
        if (n >= kVMax) {
            status = kTruncated;
            break;
        }
        prev = e;
        e = bk;
        curc[0] = Vc[0];
        curc[1] = Vc[1];
        curc[2] = Vc[2];
        if (kWide) {
            cur[0] = (TA)V[0];
            cur[1] = (TA)V[1];
            cur[2] = (TA)V[2];
        }
    }
    if (!closed && status == kOk) status = kTruncated;
    if (near) *near = any_near;
}

// Mixed form: the walk runs in the scan precision TC (solves included, as the
// plain form does), then every vertex is solved again in TS -- four lanes per
// vertex (the four Cramer determinants), eight vertices per warp instruction
// -- and every merge decision is taken again on the TS vertices.  When all
// decisions agree, the face is the TS walk's face: the same hit planes, the
// same TS vertices.  Returns false, and the caller walks again with every
// predicate and every solve in TS, when a scan met a row within 1e-6 of the
// current point other than the two it lies on (a sign or feasibility test
// near zero), when the TC walk did not close normally, took more than 32
// steps or met a vertex that is not finite in TS, or when a decision comes
// out differently in TS.
template <typename TC, typename TS, bool kGroup>
__device__ bool walk_refined(const vec4_t<TC> *rows, int ALL, const uint16_t *list, int nlist, const vec4_t<TC> &eqc,
                             const TS *eqv, const TS *p, int s, TC par_eps, TS same_eps, int lane, TS &vx, TS &vy,
                             TS &vz, int &ve, int &n, bool &closed, int8_t &status, const Grp<TC> &g)
{
    const unsigned full = 0xffffffffu;
    const TC eqf[4] = {eqc.x, eqc.y, eqc.z, eqc.w};
    const TC pf[3] = {(TC)p[0], (TC)p[1], (TC)p[2]};
    TC fx, fy, fz;
    int fve, fn, sbk, sdec, nsteps;
    bool fclosed;
    int8_t fst = kOk;
    bool near = false;
    walk<TC, TC, kGroup, TC, true>(rows, ALL, list, nlist, eqc, eqf, pf, s, par_eps, (TC)same_eps, lane, fx, fy, fz,
                                   fve, fn, fclosed, fst, sbk, sdec, nsteps, g, &near);
    if (kGroup) { // a row near a vertex in any warp's share of the scan
        if (near && lane == 0) atomicOr(&g.sh->near, 1);
        g.sync();
        near = g.sh->near != 0;
    }
    // a predicate near zero: the caller walks again with FP64 predicates
    if (near || fst != kOk || !fclosed || nsteps < 1 || nsteps > 32) return false;
    if (kGroup && g.gw != 0) return true; // the leader refines; the caller shares its outcome

    // step j's vertex in TS, into lane j
    const int G = lane >> 2, L = lane & 3, gbase = lane & ~3;
    TS rx = 0, ry = 0, rz = 0;
    bool planes_ok = true;
    for (int r0 = 0; r0 < nsteps; r0 += 8) {
        const int j = min(r0 + G, nsteps - 1);            // the step this lane group solves
        const int pb = __shfl_sync(full, sbk, j);          // its hit plane
        const int pj = __shfl_sync(full, sbk, max(j - 1, 0));
        const int pa = j == 0 ? s : pj;                    // and the edge plane it walked on
        const bool in = (unsigned)pa < (unsigned)ALL && (unsigned)pb < (unsigned)ALL;
        planes_ok = planes_ok && in;
        const TC *ra = reinterpret_cast<const TC *>(rows + (in ? pa : 0));
        const TC *rb = reinterpret_cast<const TC *>(rows + (in ? pb : 0));
        // lane t of the group converts components 2t, 2t + 1 of [row a | row b]
        const TS c0 = (TS)(L < 2 ? ra[2 * L] : rb[2 * L - 4]);
        const TS c1 = (TS)(L < 2 ? ra[2 * L + 1] : rb[2 * L - 3]);
        TS m[8];
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            m[2 * t] = __shfl_sync(full, c0, gbase | t);
            m[2 * t + 1] = __shfl_sync(full, c1, gbase | t);
        }
        const TS a00 = L == 1 ? -m[3] : m[0], a01 = L == 2 ? -m[3] : m[1], a02 = L == 3 ? -m[3] : m[2];
        const TS a10 = L == 1 ? -m[7] : m[4], a11 = L == 2 ? -m[7] : m[5], a12 = L == 3 ? -m[7] : m[6];
        const TS a20 = L == 1 ? -eqv[3] : eqv[0], a21 = L == 2 ? -eqv[3] : eqv[1], a22 = L == 3 ? -eqv[3] : eqv[2];
        const TS d = det3<TS>(a00, a01, a02, a10, a11, a12, a20, a21, a22);
        const TS x = d / __shfl_sync(full, d, gbase);
        const int src = ((lane - r0) & 7) * 4 + 1;
        const TS v0 = __shfl_sync(full, x, src), v1 = __shfl_sync(full, x, src + 1), v2 = __shfl_sync(full, x, src + 2);
        if (lane >= r0 && lane < r0 + 8) {
            rx = v0;
            ry = v1;
            rz = v2;
        }
    }
    const bool mine = lane < nsteps;
    if (!__all_sync(full, planes_ok && (!mine || (finite_bits(rx) && finite_bits(ry) && finite_bits(rz))))) return false;

    // the decisions again, on the TS vertices: step j against the last
    // vertex appended before it and, on the closing step, the first vertex
    const unsigned amask = __ballot_sync(full, mine && sdec == 0);
    const unsigned before = lane > 0 ? (amask & ((1u << lane) - 1u)) : 0u;
    const int la = before ? 31 - __clz(before) : 0;
    const TC Vc[3] = {(TC)rx, (TC)ry, (TC)rz};
    const TC lx = __shfl_sync(full, Vc[0], la), ly = __shfl_sync(full, Vc[1], la), lz = __shfl_sync(full, Vc[2], la);
    const TC f0 = __shfl_sync(full, Vc[0], 0), f1 = __shfl_sync(full, Vc[1], 0), f2 = __shfl_sync(full, Vc[2], 0);
    const bool check = mine && lane > 0;
    int s1 = same_filter<TC, TS>(Vc, lx, ly, lz, same_eps);
    int s2 = sbk == s ? same_filter<TC, TS>(Vc, f0, f1, f2, same_eps) : 0;
    if (__any_sync(full, check && (s1 < 0 || (s1 == 0 && s2 < 0)))) {
        const TS Lx = __shfl_sync(full, rx, la), Ly = __shfl_sync(full, ry, la), Lz = __shfl_sync(full, rz, la);
        const TS Fx = __shfl_sync(full, rx, 0), Fy = __shfl_sync(full, ry, 0), Fz = __shfl_sync(full, rz, 0);
        if (check && s1 < 0) s1 = (fabs(rx - Lx) + fabs(ry - Ly) + fabs(rz - Lz) < same_eps) ? 1 : 0;
        if (check && s2 < 0) s2 = (fabs(rx - Fx) + fabs(ry - Fy) + fabs(rz - Fz) < same_eps) ? 1 : 0;
    }
    const int dec = s1 == 1 ? 1 : (sbk == s && s2 == 1 ? 2 : 0);
    if (!__all_sync(full, !check || dec == sdec)) return false;

    // vertex o is the o-th appended step; its edge is the hit plane of the
    // last step before the next append, a closing merge excepted
    n = __popc(amask);
    const int so = lane < n ? (int)__fns(amask, 0, lane + 1) : 0;
    const int snext = lane + 1 < n ? (int)__fns(amask, 0, lane + 2) : nsteps;
    int kl = (snext - 1) & 31;
    if (__shfl_sync(full, sdec, kl) == 2) kl = (kl - 1) & 31;
    const int e_out = __shfl_sync(full, sbk, kl);
    const TS ox = __shfl_sync(full, rx, so), oy = __shfl_sync(full, ry, so), oz = __shfl_sync(full, rz, so);
    if (lane < n) {
        vx = ox;
        vy = oy;
        vz = oz;
        ve = e_out;
    } else {
        vx = vy = vz = TS(0);
        ve = -1;
    }
    closed = true;
    status = kOk;
    return true;
}

// Row pruning before the walk.  The face polygon is the intersection of the
// half-planes the rows cut out of the face plane.  In coordinates u of that
// plane centred on the start point p, row k reads m_k . u <= c_k, with
// c_k = -(w_k . p + b_k) the distance from p to the row's plane (the rows are
// normalised) and m_k the in-plane part of w_k.  For c_k > 0 the row's dual
// point q_k = m_k / c_k lies strictly inside the convex hull of the other dual
// points and the origin exactly when the row's line misses the polygon (the
// polar of a polygon around p): such a row is never the first plane the walk
// hits on an edge.  A sample of the rows (every eighth) gives, for eight
// directions, the extreme dual points; their convex polygon lies inside that
// hull, and so does the circle of radius r around the origin inscribed in it.
// Every row whose dual point lies inside 0.98 r -- computed with c_k lowered
// by a bound on its rounding -- is dropped, and the walk scans the kept rows
// only, so its decisions (the first hit, ties to the lower row) are those of
// the scan over every row.  Rows through or near p and rows that are not
// finite are always kept; the sample uses only rows with c_k well above the
// rounding bound, so that its dual points are accurate.  Returns the number
// of kept rows (their indices in sh->list), or -1 -- the walk scans every
// row -- when the sample gives no circle or more than kListCap rows are kept.
template <typename TC, bool kGroup>
__device__ int prune_rows(const vec4_t<TC> *rows, int ALL, const vec4_t<TC> &eqc, const TC *pc, int lane,
                          const Grp<TC> &g)
{
    const unsigned full = 0xffffffffu;
    GroupShared<TC> *sh = g.sh;
    const int w = kGroup ? g.gw : 0, G = kGroup ? g.G : 1;
    // orthonormal basis (e1, e2) of the face plane
    TC nx = eqc.x, ny = eqc.y, nz = eqc.z;
    const TC nn = nx * nx + ny * ny + nz * nz;
    if (!(nn > TC(0)) || !finite_bits(nn)) return -1; // uniform: every lane reads the same plane
    const TC inv = rsqrt(nn);
    nx *= inv;
    ny *= inv;
    nz *= inv;
    const TC ax = (fabs(nx) <= fabs(ny) && fabs(nx) <= fabs(nz)) ? TC(1) : TC(0);
    const TC ay = (ax == TC(0) && fabs(ny) <= fabs(nz)) ? TC(1) : TC(0);
    const TC az = (ax == TC(0) && ay == TC(0)) ? TC(1) : TC(0);
    TC e1x = ay * nz - az * ny, e1y = az * nx - ax * nz, e1z = ax * ny - ay * nx;
    const TC i1 = rsqrt(e1x * e1x + e1y * e1y + e1z * e1z);
    e1x *= i1;
    e1y *= i1;
    e1z *= i1;
    const TC e2x = ny * e1z - nz * e1y, e2y = nz * e1x - nx * e1z, e2z = nx * e1y - ny * e1x;
    const TC p0 = pc[0], p1 = pc[1], p2 = pc[2];
    // rounding of c_k in TC, and the sample's floor on c_k
    const TC dc = (sizeof(TC) == 4 ? TC(1e-6) : TC(1e-14)) * (TC(1) + fabs(p0) + fabs(p1) + fabs(p2));
    const TC cmin = TC(1000) * dc;
    if (w == 0 && lane == 0) sh->nlist = 0;

    // sample: the extreme dual point in directions 0, 45, ..., 315 degrees
    TC bv[8];
    int bi[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        bv[m] = TC(-INFINITY);
        bi[m] = 0x7fffffff;
    }
    for (int k = 8 * (32 * w + lane); k < ALL; k += 8 * 32 * G) {
        const vec4_t<TC> r = rows[k];
        const TC c = -(r.x * p0 + r.y * p1 + r.z * p2 + r.w);
        if (!(c >= cmin) || !finite_bits(c)) continue;
        const TC ic = TC(1) / c;
        const TC qx = (r.x * e1x + r.y * e1y + r.z * e1z) * ic;
        const TC qy = (r.x * e2x + r.y * e2y + r.z * e2z) * ic;
        const TC v[8] = {qx, qx + qy, qy, qy - qx, -qx, -qx - qy, -qy, qx - qy};
#pragma unroll
        for (int m = 0; m < 8; ++m)
            if (v[m] > bv[m]) {
                bv[m] = v[m];
                bi[m] = k;
            }
    }
#pragma unroll
    for (int m = 0; m < 8; ++m)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const TC ov = __shfl_xor_sync(full, bv[m], o);
            const int oi = __shfl_xor_sync(full, bi[m], o);
            if (ov > bv[m] || (ov == bv[m] && oi < bi[m])) {
                bv[m] = ov;
                bi[m] = oi;
            }
        }
    if (kGroup) {
        if (lane < 8) {
            TC v = bv[0];
            int i = bi[0];
#pragma unroll
            for (int m = 1; m < 8; ++m)
                if (lane == m) v = bv[m], i = bi[m];
            sh->ext.v[w][lane] = v;
            sh->ext.i[w][lane] = (int16_t)(i == 0x7fffffff ? -1 : i);
        }
        g.sync();
#pragma unroll
        for (int m = 0; m < 8; ++m) {
            bv[m] = TC(-INFINITY);
            bi[m] = 0x7fffffff;
            for (int u = 0; u < G; ++u) {
                const TC ov = sh->ext.v[u][m];
                const int oi = sh->ext.i[u][m] < 0 ? 0x7fffffff : (int)sh->ext.i[u][m];
                if (ov > bv[m] || (ov == bv[m] && oi < bi[m])) {
                    bv[m] = ov;
                    bi[m] = oi;
                }
            }
        }
        g.sync(); // every warp has read the extremes: the list may overwrite them
    }
    // the extreme points in counter-clockwise order (lane m < 8: direction
    // m), and the radius of the circle around the origin inscribed in their
    // polygon: the smallest distance from the origin to an edge, which must
    // have the origin strictly on its left
    bool ok = true;
#pragma unroll
    for (int m = 0; m < 8; ++m) ok = ok && bi[m] != 0x7fffffff;
    if (!ok) return -1; // a direction without a sampled row: the polygon may be open that way
    int mine = bi[0];
#pragma unroll
    for (int m = 1; m < 8; ++m)
        if ((lane & 7) == m) mine = bi[m];
    const vec4_t<TC> er = rows[mine];
    const TC eic = TC(1) / -(er.x * p0 + er.y * p1 + er.z * p2 + er.w);
    const TC qx = (er.x * e1x + er.y * e1y + er.z * e1z) * eic;
    const TC qy = (er.x * e2x + er.y * e2y + er.z * e2z) * eic;
    const int nxt = (lane + 1) & 7;
    const TC qx1 = __shfl_sync(full, qx, nxt), qy1 = __shfl_sync(full, qy, nxt);
    const int bi1 = __shfl_sync(full, mine, nxt);
    const bool edge = lane < 8 && bi1 != mine;
    const TC dx = qx1 - qx, dy = qy1 - qy;
    const TC cr = dy * qx - dx * qy; // (E1 - E0) x (O - E0)
    const TC len = sqrt(dx * dx + dy * dy);
    const bool bad = edge && !(cr > TC(0) && len > TC(0));
    TC rad = edge && !bad ? cr / len : TC(INFINITY);
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) rad = fmin(rad, __shfl_xor_sync(full, rad, o));
    rad = __shfl_sync(full, rad, 0);
    const int edges = __popc(__ballot_sync(full, edge));
    if (__any_sync(full, bad) || edges < 3 || !(rad > TC(0)) || !finite_bits(rad)) return -1;
    const TC re = TC(0.98) * rad;
    const TC re2 = re * re;

    // every row: keep those whose dual point may lie outside the circle
    for (int k0 = 32 * w; k0 < ALL; k0 += 32 * G) {
        const int k = k0 + lane;
        bool keep = false;
        if (k < ALL) {
            const vec4_t<TC> r = rows[k];
            const TC c = -(r.x * p0 + r.y * p1 + r.z * p2 + r.w) - dc;
            const TC m1 = r.x * e1x + r.y * e1y + r.z * e1z;
            const TC m2 = r.x * e2x + r.y * e2y + r.z * e2z;
            keep = !(c > TC(0)) || !(m1 * m1 + m2 * m2 < re2 * c * c);
        }
        const unsigned b = __ballot_sync(full, keep);
        if (b) {
            int base = 0;
            if (lane == 0) base = atomicAdd(&sh->nlist, __popc(b));
            base = __shfl_sync(full, base, 0);
            const int pos = base + __popc(b & ((1u << lane) - 1u));
            if (keep && pos < kListCap) sh->list[pos] = (uint16_t)k;
        }
    }
    if (kGroup)
        g.sync();
    else
        __syncwarp();
    const int nl = sh->nlist;
    return nl <= kListCap ? nl : -1;
}

// Rows are staged normalised (|w| = 1, zero rows become 0.x + sign(b) inf):
// signed geometric distances are then plain dot products, the same quantity
// the reference's feasibility test computes as (w.x + b) * rsqrt(|w|^2)
// (kernel.h:729-795).  TC is the scan precision, TS the solve precision.
template <typename TC, typename TS, bool kGroup>
__global__ void __launch_bounds__(256, 3) polygon_kernel(NetDev net, RegionsDev reg, ChunkDev ch, HashDev hs, Tolerances tol,
                                                      int G_, int prune, unsigned long long *nfp64, int *err)
{
    const int G = kGroup ? G_ : 1;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const int F = (blockDim.x >> 5) / G; // faces per block
    const int gid = wib / G;
    const int ALL = net.ALL;
    const int N = net.N;
    const int W = net.W;
    vec4_t<TC> *rows = reinterpret_cast<vec4_t<TC> *>(smem_raw) + (size_t)gid * net.ALLP;
    Grp<TC> g;
    g.G = G;
    g.gw = wib % G;
    g.bar = 1 + gid;
    g.sh = reinterpret_cast<GroupShared<TC> *>(smem_raw + (size_t)F * net.ALLP * sizeof(vec4_t<TC>) +
                                               (size_t)gid * group_shared_bytes<TC>());
    // (the group's shared block also holds the pruning list: one per face)
    const TC eps = (TC)tol.eps, par_eps = (TC)tol.par_eps;
    const TS same_eps = (TS)tol.same_eps;

    long long head;
    int count;
    chunk_range(ch, head, count);
    // a region per group: by launch position, or (fixed grid of the
    // graph-driven loop) from the wave's work counter; the leader takes it
    // and the group reads it from shared memory
    long long rl_next = (long long)blockIdx.x * F + gid;
    if (g.gw == 0 && lane == 0) {
        umma::mbar_init(&g.sh->rbar, 1);
        umma::fence_mbar_init();
    }
    uint32_t rphase = 0; // faces taken by this group: the row barrier's phase
    for (;;) {
        long long rl;
        if (g.gw == 0) {
            rl = ch.ctl ? next_work(ch.ctl, lane) : rl_next;
            if (kGroup && lane == 0) {
                g.sh->rl = rl;
                g.sh->near = 0;
            }
        }
        rl_next += (long long)gridDim.x * F;
        if (kGroup) {
            g.sync();
            rl = g.sh->rl;
        }
        if (rl >= count) break;
        const long long rid = head + rl;
        const vec4_t<TC> *grows = reinterpret_cast<const vec4_t<TC> *>((const TC *)ch.cons + (size_t)rl * net.ALLP * 4);
        // the region's rows into shared memory by one bulk copy (the leader
        // issues it once every warp of the group is done with the previous
        // face's rows), then normalised in place
        {
            const uint32_t rbytes = (uint32_t)ALL * (uint32_t)sizeof(vec4_t<TC>);
            if (!kGroup) __syncwarp(); // (a group has met at its barrier above)
            if (g.gw == 0 && lane == 0) {
                umma::fence_proxy_async(); // earlier generic reads of the rows before the copy's writes
                umma::mbar_expect_tx(&g.sh->rbar, rbytes);
                umma::bulk_g2s(rows, grows, rbytes, &g.sh->rbar);
            }
            if (!umma::mbar_wait(&g.sh->rbar, rphase & 1u, kRowWaitIters)) {
                atomicOr(err, kErrWait);
                umma::mbar_wait(&g.sh->rbar, rphase & 1u, kRowWaitIters); // nothing lands after the face is left
            }
            ++rphase;
        }
        for (int q = 32 * g.gw + lane; q < ALL; q += 32 * G) {
            vec4_t<TC> v = rows[q];
            const TC n2 = v.x * v.x + v.y * v.y + v.z * v.z;
            if (n2 > TC(0)) {
                const TC inv = rsqrt(n2); // as the reference's distance normalisation
                v.x *= inv;
                v.y *= inv;
                v.z *= inv;
                v.w *= inv;
            } else {
                v.w = v.w > TC(0) ? TC(INFINITY) : (v.w < TC(0) ? TC(-INFINITY) : TC(NAN));
            }
            rows[q] = v;
        }
        if (kGroup)
            g.sync();
        else
            __syncwarp();
        TS eqv[4];
        const vec4_t<TC> eqc = ld4<TC>((const TC *)ch.eq + (size_t)rl * 4); // scan precision copy
        eqv[0] = (TS)eqc.x;
        eqv[1] = (TS)eqc.y;
        eqv[2] = (TS)eqc.z;
        eqv[3] = (TS)eqc.w;
        const TS *midp = (const TS *)reg.mid + (size_t)rid * 4;
        TS p[3] = {midp[0], midp[1], midp[2]};
        int s = reg.start[rid];
        const bool is_seed = (s < 0);
        int8_t status = kOk;

        // ---------------------------------------------------- seed start search
        if (is_seed) {
            // pairs x <= 812 reach sorted positions up to 56: keep the 64 nearest,
            // position q in lane q % 32, register q / 32.  In a group, every
            // selection pass splits the rows over the warps (the partial
            // choices meet in shared memory), and the warps test G pairs at a
            // time, the smallest feasible x winning (measured on GB300: with
            // every warp repeating the whole search, the seeds of a 4,096-row
            // network took a whole wave's time)
            const int ksel = ALL < kTopK ? ALL : kTopK;
            const int k0 = kGroup ? 32 * g.gw + lane : lane, ks = kGroup ? 32 * G : 32;
            int top0 = -1, top1 = -1;
            unsigned long long pk = ~0ull;
            int pi = -1;
            const TC pc[3] = {(TC)p[0], (TC)p[1], (TC)p[2]};
            for (int sel = 0; sel < ksel; ++sel) {
                unsigned long long bk = 0ull;
                int bi = 0x7fffffff;
                for (int k = k0; k < ALL; k += ks) {
                    const vec4_t<TC> v = rows[k];
                    const TC d = v.x * pc[0] + v.y * pc[1] + v.z * pc[2] + v.w;
                    const unsigned long long key = order_key<TC>(d);
                    const bool below = key < pk || (key == pk && k > pi);
                    if (below && ahead(key, k, bk, bi)) {
                        bk = key;
                        bi = k;
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    const unsigned long long ok = __shfl_xor_sync(0xffffffffu, bk, o);
                    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
                    if (ahead(ok, oi, bk, bi)) {
                        bk = ok;
                        bi = oi;
                    }
                }
                if (kGroup) {
                    const int par = sel & 1;
                    if (lane == 0) {
                        g.sh->seed.sk[par][g.gw] = bk;
                        g.sh->bk[par][g.gw] = bi;
                    }
                    g.sync();
                    bk = g.sh->seed.sk[par][0];
                    bi = g.sh->bk[par][0];
                    for (int w = 1; w < G; ++w)
                        if (ahead(g.sh->seed.sk[par][w], g.sh->bk[par][w], bk, bi)) {
                            bk = g.sh->seed.sk[par][w];
                            bi = g.sh->bk[par][w];
                        }
                }
                if (lane == (sel & 31)) {
                    if (sel < 32) top0 = bi;
                    else top1 = bi;
                }
                pk = bk;
                pi = bi;
            }
            int x_max = (ALL - 1) * (ALL - 2);
            if (x_max > 812) x_max = 812;
            if (x_max < 0) x_max = 0;
            s = -1;
            for (int xb = 0, round = 0; xb <= x_max; xb += G, ++round) {
                const int x = xb + (kGroup ? g.gw : 0);
                bool good = false;
                TS v[3];
                int ri = -1;
                if (x <= x_max) {
                    int i, j;
                    get_i_j(x, ALL, i, j);
                    const int ri0 = __shfl_sync(0xffffffffu, top0, i & 31), ri1 = __shfl_sync(0xffffffffu, top1, i & 31);
                    const int rj0 = __shfl_sync(0xffffffffu, top0, j & 31), rj1 = __shfl_sync(0xffffffffu, top1, j & 31);
                    ri = i < 32 ? ri0 : ri1;
                    const int rj = j < 32 ? rj0 : rj1;
                    TC vc[3];
                    warp_solve<TC, TS>(rows, ri, rj, eqv, v, vc, lane);
                    bool bad = false;
                    for (int k = lane; k < ALL; k += 32) {
                        if (k == ri || k == rj) continue;
                        const vec4_t<TC> r = rows[k];
                        if (r.x * vc[0] + r.y * vc[1] + r.z * vc[2] + r.w > eps) bad = true;
                    }
                    good = !__any_sync(0xffffffffu, bad);
                }
                if (kGroup) { // the smallest feasible pair of the round, from its warp
                    const int par = (round + ksel) & 1; // not the last selection pass's slots
                    // (a warp still reading those may lag one barrier behind)
                    if (lane == 0) g.sh->bk[par][g.gw] = good ? x : 0x7fffffff;
                    g.sync();
                    int xw = 0x7fffffff;
                    for (int w = 0; w < G; ++w) xw = min(xw, g.sh->bk[par][w]);
                    if (xw == 0x7fffffff) continue;
                    if (good && x == xw && lane == 0) {
                        g.sh->seed.sri = ri;
                        g.sh->seed.sv[0] = (double)v[0];
                        g.sh->seed.sv[1] = (double)v[1];
                        g.sh->seed.sv[2] = (double)v[2];
                    }
                    g.sync();
                    s = g.sh->seed.sri;
                    p[0] = (TS)g.sh->seed.sv[0];
                    p[1] = (TS)g.sh->seed.sv[1];
                    p[2] = (TS)g.sh->seed.sv[2];
                    g.sync(); // read by every warp before the pruning may overwrite it
                    break;
                }
                if (good) {
                    s = ri;
                    p[0] = v[0];
                    p[1] = v[1];
                    p[2] = v[2];
                    break;
                }
            }
            if (s < 0) status = kNoStart;
        }

        // ---------------------------------------------------- row pruning
        int nlist = -1;
        const uint16_t *list = nullptr;
        if (s >= 0 && prune && ALL >= kPruneMin) {
            const TC pc3[3] = {(TC)p[0], (TC)p[1], (TC)p[2]};
            nlist = prune_rows<TC, kGroup>(rows, ALL, eqc, pc3, lane, g);
            if (nlist >= 0) list = g.sh->list;
        }

        // ---------------------------------------------------- walk
        // lane i holds vertex i and the plane of the edge leaving it
        TS vx = 0, vy = 0, vz = 0;
        int ve = -1;
        int n = 0;
        bool closed = false;
        if (s >= 0) {
            bool done = false;
            if (sizeof(TS) > sizeof(TC)) // scan-precision walk, vertices refined in the solve precision
            {
                done = walk_refined<TC, TS, kGroup>(rows, ALL, list, nlist, eqc, eqv, p, s, par_eps, same_eps, lane, vx,
                                                    vy, vz, ve, n, closed, status, g);
                if (kGroup) { // the leader's outcome for the group
                    if (g.gw == 0 && lane == 0) g.sh->done = done ? 1 : 0;
                    g.sync();
                    done = g.sh->done != 0;
                }
            }
            if (!done) {
                int sbk, sdec, nsteps;
                if (sizeof(TS) > sizeof(TC)) { // mixed form: FP64 predicates and FP64 solves
                    if (g.gw == 0 && lane == 0) atomicAdd(nfp64, 1ull);
                    walk<TC, TS, kGroup, TS, false>(rows, ALL, list, nlist, eqc, eqv, p, s, par_eps, same_eps, lane, vx,
                                                    vy, vz, ve, n, closed, status, sbk, sdec, nsteps, g);
                } else {
                    walk<TC, TS, kGroup>(rows, ALL, list, nlist, eqc, eqv, p, s, par_eps, same_eps, lane, vx, vy, vz, ve,
                                         n, closed, status, sbk, sdec, nsteps, g);
                }
            }
        }
        const bool leader = !kGroup || g.gw == 0;

        // ---------------------------------------------------- outputs
        if (leader && lane == 0) { // the leader writes the face
            reg.nv[rid] = n;
            reg.status[rid] = status;
        }
        if (leader && lane < n) {
            TS *vo = (TS *)reg.verts + ((size_t)rid * kVMax + lane) * 3;
            vo[0] = vx;
            vo[1] = vy;
            vo[2] = vz;
            reg.edges[(size_t)rid * kVMax + lane] = ve;
        }

        // ---------------------------------------------------- neighbours
        // the plane crossed by edge `lane` where a neighbour is to be
        // inserted (else -1), published by the leader; warp gw of the group
        // inserts the neighbours of the edges lane = gw (mod G), one after
        // the other, each by the whole warp (measured on GB300: with the
        // leader inserting all of them the other warps waited at the next
        // face's barrier)
        int kv = -1;
        if (leader && lane < n && ve >= 0 && ve < N && (closed || lane < n - 1) && !(!is_seed && ve == s)) kv = ve;
        if (kGroup) {
            if (list) g.sync(); // every warp's walk has done with the pruning list
            if (g.gw == 0) g.sh->ve[lane] = kv;
            g.sync();
            kv = g.sh->ve[lane];
        }
        const bool mine = !kGroup || lane % G == g.gw;
        int rec = -1;
        const uint32_t *pkey = reg.keys + (size_t)rid * W;
        unsigned todo = __ballot_sync(0xffffffffu, mine && kv >= 0);
        const uint64_t phash = reg.hash[rid];
        while (todo) {
            const int src = __ffs(todo) - 1;
            todo &= todo - 1u;
            const int k = __shfl_sync(0xffffffffu, kv, src);
            const int got = warp_insert(reg, hs, head, ALL, W, pkey, phash, rl, k, lane, err);
            if (lane == src) rec = got;
        }
        if (mine && lane < kVMax) ch.rec[(size_t)rl * kVMax + lane] = rec;
        __syncwarp();
    }
}

} // namespace

// Faces per block for G warps per face: as many as keep a block's rows
// (and each face's shared block) within 73 KB (three blocks per SM), at most
// 8 / G, a power of two.
int polygon_faces_per_block(size_t face_bytes, int G)
{
    int F = 1;
    while (2 * F * G <= 8 && (size_t)(2 * F) * face_bytes <= 73u * 1024u) F *= 2;
    return F;
}

// Automatic warps per face: eight warps per block, split between faces
// and the warps of a face as the rows allow.
int polygon_face_warps(int prec, int ALLP)
{
    const size_t face_bytes = prec == kFloat64 ? sizeof(double4) * (size_t)ALLP + group_shared_bytes<double>()
                                               : sizeof(float4) * (size_t)ALLP + group_shared_bytes<float>();
    const int F = polygon_faces_per_block(face_bytes, 1);
    return 8 / F;
}

template <typename TC, typename TS>
void launch_one(const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, const HashDev &hs, const Tolerances &tol,
                int *d_err, int G, int prune, unsigned long long *nfp64, cudaStream_t st)
{
    const size_t row_bytes = sizeof(vec4_t<TC>) * (size_t)net.ALLP;
    const int F = polygon_faces_per_block(row_bytes + group_shared_bytes<TC>(), G);
    const size_t smem = (row_bytes + group_shared_bytes<TC>()) * F;
    auto k = G > 1 ? polygon_kernel<TC, TS, true> : polygon_kernel<TC, TS, false>;
    if (smem > 48 * 1024) cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int sms = device_sms();
    const int threads = 32 * F * G;
    int grid;
    if (ch.ctl) { // wave size on the device: as many blocks as stay resident
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, threads, smem);
        grid = sms * std::max(per_sm, 1);
    } else {
        const long long need = (ch.count + F - 1) / F;
        grid = (int)std::min<long long>(need, (long long)sms * 16);
    }
    k<<<grid, threads, smem, st>>>(net, reg, ch, hs, tol, G, prune, nfp64, d_err);
}

void launch_polygon(int prec, const NetDev &net, const RegionsDev &reg, const ChunkDev &ch, const HashDev &hs,
                    const Tolerances &tol, int face_warps, int prune, unsigned long long *nfp64, int *d_err,
                    cudaStream_t st)
{
    if (!ch.ctl && ch.count <= 0) return;
    const int G = face_warps > 0 ? face_warps : polygon_face_warps(prec, net.ALLP);
    if (prec == kFloat64)
        launch_one<double, double>(net, reg, ch, hs, tol, d_err, G, prune, nfp64, st);
    else if (prec == kMixed)
        launch_one<float, double>(net, reg, ch, hs, tol, d_err, G, prune, nfp64, st);
    else
        launch_one<float, float>(net, reg, ch, hs, tol, d_err, G, prune, nfp64, st);
}

} // namespace am
