/*
 * am_oracle_impl.h -- type-generic body of the CPU restatement (test
 * infrastructure only, see am_oracle.h).  Included by am_oracle.c once per
 * arithmetic type with REAL / SFX / R_EPS / R_SAME_EPS / R_PH_MUL defined.
 *
 * Every function cites the reference line range it restates (paths relative
 * to the reference project root).
 */

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* r_sqrt, kernel.h:33-34: 1/sqrt in the working precision */
static inline REAL FN(rsq)(REAL x) { return (REAL)1 / CAT(amo_sqrt, SFX)(x); }

static inline REAL FN(mask_of)(const uint32_t *bits, int k) { return (REAL)((bits[k >> 5] >> (k & 31)) & 1u); }

/* DET_3x3 macro, backend/inc/kernel.h:509 */
#define AMO_DET(a0, a1, a2, a3, a4, a5, a6, a7, a8) \
    ((a0) * ((a4) * (a8) - (a5) * (a7)) - (a1) * ((a3) * (a8) - (a5) * (a6)) + (a2) * ((a3) * (a7) - (a4) * (a6)))

/* solve_3x3, backend/inc/kernel.h:553-571 (the fp64-promotion variant is
 * compiled out by macro.h:11) -- Cramer's rule for A x + b = 0. */
static void FN(solve3)(const REAL *A, const REAL *b, REAL *x)
{
    REAL d0 = AMO_DET(A[0], A[1], A[2], A[3], A[4], A[5], A[6], A[7], A[8]);
    REAL d1 = AMO_DET((-b[0]), A[1], A[2], (-b[1]), A[4], A[5], (-b[2]), A[7], A[8]);
    REAL d2 = AMO_DET(A[0], (-b[0]), A[2], A[3], (-b[1]), A[5], A[6], (-b[2]), A[8]);
    REAL d3 = AMO_DET(A[0], A[1], (-b[0]), A[3], A[4], (-b[1]), A[6], A[7], (-b[2]));
    x[0] = d1 / d0;
    x[1] = d2 / d0;
    x[2] = d3 / d0;
}

/* net view: offsets of every linear layer's output rows (mlp.h:40-50) */
typedef struct {
    const amo_net *net;
    int N, E, all, maxw;
    int offs[64];
} FN(amo_view);

/* fill_constraints for one region, backend/inc/process.h:18-193, followed by
 * offset_b_equ (process.h:198-203). */
static void FN(compose)(const FN(amo_view) *v, const uint32_t *bits, REAL iso,
                        REAL *w_in, REAL *b_in, REAL *w_eq, REAL *b_eq, REAL *wt, REAL *bt)
{
    const amo_net *net = v->net;
    const int *nodes = net->nodes;
    const int N = v->N;
    const int n_lin = net->n_lin;
    int i, r, c, m;

    /* layer-0 rows: cudaMemcpyStrided_D2D of weights[0] / biases[0], process.h:36-39 */
    {
        const REAL *W0 = (const REAL *)net->W[0];
        const REAL *b0 = (const REAL *)net->b[0];
        for (r = 0; r < nodes[1]; ++r) {
            for (c = 0; c < 3; ++c) w_in[3 * r + c] = W0[3 * r + c];
            b_in[r] = b0[r];
        }
    }

    /* hidden layers, process.h:41-149 */
    for (i = 1; i < n_lin - 1; ++i) {
        const int so = v->offs[i];
        const int sd = nodes[i];
        const int prev = so - sd;
        const int nout = nodes[i + 1];
        const REAL *Wi = (const REAL *)net->W[i];
        const REAL *bi = (const REAL *)net->b[i];
        /* cudaMaskRowsStrided<3>/<1>, process.h:48-57 */
        for (r = 0; r < sd; ++r) {
            REAL mk = FN(mask_of)(bits, prev + r);
            for (c = 0; c < 3; ++c) wt[3 * r + c] = w_in[3 * (prev + r) + c] * mk;
            bt[r] = b_in[prev + r] * mk;
        }
        /* cublasMatMulBatched / cublasMatVecMulAddBatched, process.h:60-70 */
        for (m = 0; m < nout; ++m) {
            const REAL *wr = Wi + (size_t)m * sd;
            REAL a0 = 0, a1 = 0, a2 = 0, ab = 0;
            for (r = 0; r < sd; ++r) {
                a0 += wr[r] * wt[3 * r + 0];
                a1 += wr[r] * wt[3 * r + 1];
                a2 += wr[r] * wt[3 * r + 2];
                ab += wr[r] * bt[r];
            }
            w_in[3 * (so + m) + 0] = a0;
            w_in[3 * (so + m) + 1] = a1;
            w_in[3 * (so + m) + 2] = a2;
            b_in[so + m] = ab + bi[m];
        }
        /* additive skip connections, process.h:73-146 */
        {
            const int *row = net->arc_table + (size_t)(i - 1) * net->arc_cols;
            int ci;
            for (ci = 0; ci < row[0]; ++ci) {
                const int from = row[1 + 2 * ci];
                const int t = row[2 + 2 * ci];
                const int th = net->tm_shape[2 * t], tw = net->tm_shape[2 * t + 1];
                const REAL *T = (const REAL *)net->tm[t];
                if (th == 0 && tw == 0) {
                    if (from == 0) { /* cudaAddIdentityBatched, process.h:89-91 */
                        for (c = 0; c < 3; ++c) w_in[3 * (so + c) + c] += (REAL)1;
                    } else { /* cudaMaskRowsAddStrided, process.h:95-104 */
                        const int os = v->offs[from - 1];
                        const int dec = nodes[from];
                        for (r = 0; r < dec; ++r) {
                            REAL mk = FN(mask_of)(bits, os + r);
                            for (c = 0; c < 3; ++c) w_in[3 * (so + r) + c] = w_in[3 * (so + r) + c] + w_in[3 * (os + r) + c] * mk;
                            b_in[so + r] = b_in[so + r] + b_in[os + r] * mk;
                        }
                    }
                } else {
                    if (from == 0) { /* cudaMatAddBatched, process.h:111-114 */
                        int e;
                        for (e = 0; e < th * tw; ++e) w_in[3 * so + e] = w_in[3 * so + e] + T[e];
                    } else { /* mask + beta=1 GEMMs, process.h:119-142 */
                        const int os = v->offs[from - 1];
                        const int dec = nodes[from];
                        for (r = 0; r < dec; ++r) {
                            REAL mk = FN(mask_of)(bits, os + r);
                            for (c = 0; c < 3; ++c) wt[3 * r + c] = w_in[3 * (os + r) + c] * mk;
                            bt[r] = b_in[os + r] * mk;
                        }
                        for (m = 0; m < th; ++m) {
                            const REAL *tr = T + (size_t)m * dec;
                            REAL a0 = 0, a1 = 0, a2 = 0, ab = 0;
                            for (r = 0; r < dec; ++r) {
                                a0 += tr[r] * wt[3 * r + 0];
                                a1 += tr[r] * wt[3 * r + 1];
                                a2 += tr[r] * wt[3 * r + 2];
                                ab += tr[r] * bt[r];
                            }
                            w_in[3 * (so + m) + 0] += a0;
                            w_in[3 * (so + m) + 1] += a1;
                            w_in[3 * (so + m) + 2] += a2;
                            b_in[so + m] = ab + b_in[so + m];
                        }
                    }
                }
            }
        }
    }

    /* output layer -> face plane, process.h:151-178 */
    {
        const int so = v->offs[i];
        const int sd = nodes[i];
        const int prev = so - sd;
        const REAL *WL = (const REAL *)net->W[i];
        const REAL *bL = (const REAL *)net->b[i];
        REAL a0 = 0, a1 = 0, a2 = 0, ab = 0;
        for (r = 0; r < sd; ++r) {
            REAL mk = FN(mask_of)(bits, prev + r);
            wt[3 * r + 0] = w_in[3 * (prev + r) + 0] * mk;
            wt[3 * r + 1] = w_in[3 * (prev + r) + 1] * mk;
            wt[3 * r + 2] = w_in[3 * (prev + r) + 2] * mk;
            bt[r] = b_in[prev + r] * mk;
        }
        for (r = 0; r < sd; ++r) {
            a0 += WL[r] * wt[3 * r + 0];
            a1 += WL[r] * wt[3 * r + 1];
            a2 += WL[r] * wt[3 * r + 2];
            ab += WL[r] * bt[r];
        }
        w_eq[0] = a0;
        w_eq[1] = a1;
        w_eq[2] = a2;
        *b_eq = ab + bL[0];
        /* Connections into the output layer: the reference's loop stops at
         * fc_layers_num - 2 (process.h:42) and never adds them.  Only applied
         * when output_skips != 0 (not the reference's behaviour). */
        if (net->output_skips && n_lin >= 2) {
            const int *row = net->arc_table + (size_t)(n_lin - 2) * net->arc_cols;
            int ci;
            for (ci = 0; ci < row[0]; ++ci) {
                const int from = row[1 + 2 * ci];
                const int t = row[2 + 2 * ci];
                const int th = net->tm_shape[2 * t], tw = net->tm_shape[2 * t + 1];
                const REAL *T = (const REAL *)net->tm[t];
                if (th == 0 && tw == 0) {
                    if (from != 0 && nodes[from] == 1) {
                        const int os = v->offs[from - 1];
                        REAL mk = FN(mask_of)(bits, os);
                        for (c = 0; c < 3; ++c) w_eq[c] += w_in[3 * os + c] * mk;
                        *b_eq += b_in[os] * mk;
                    }
                } else if (from == 0) {
                    for (c = 0; c < 3; ++c) w_eq[c] += T[c];
                } else {
                    const int os = v->offs[from - 1];
                    const int dec = nodes[from];
                    REAL s0 = 0, s1 = 0, s2 = 0, sb = 0;
                    for (r = 0; r < dec; ++r) {
                        REAL mk = FN(mask_of)(bits, os + r);
                        s0 += T[r] * (w_in[3 * (os + r) + 0] * mk);
                        s1 += T[r] * (w_in[3 * (os + r) + 1] * mk);
                        s2 += T[r] * (w_in[3 * (os + r) + 2] * mk);
                        sb += T[r] * (b_in[os + r] * mk);
                    }
                    w_eq[0] += s0;
                    w_eq[1] += s1;
                    w_eq[2] += s2;
                    *b_eq += sb;
                }
            }
        }
    }

    /* cudaSignConstraints<3>/<1>, process.h:181-186: active units become -(w.x+b) <= 0 */
    for (r = 0; r < N; ++r) {
        REAL sg = (REAL)(1.0 - 2.0 * (double)FN(mask_of)(bits, r));
        for (c = 0; c < 3; ++c) w_in[3 * r + c] *= sg;
        b_in[r] *= sg;
    }
    /* extra constraints, process.h:189-192 */
    {
        const REAL *we = (const REAL *)net->w_extra;
        const REAL *be = (const REAL *)net->b_extra;
        for (r = 0; r < v->E; ++r) {
            for (c = 0; c < 3; ++c) w_in[3 * (N + r) + c] = we[3 * r + c];
            b_in[N + r] = be[r];
        }
    }
    /* offset_b_equ, process.h:198-203 */
    *b_eq -= iso;
}

/* fill_distance (process.h:208-239, DistanceIn3D) + sortDistance
 * (process.h:244-264): indices ordered by descending signed geometric
 * distance, ties by ascending index (two stable sorts).  NaN distances
 * (zero rows with zero bias) are ordered last; the reference leaves their
 * position to thrust's merge sort. */
static void FN(sort_dist)(int all, const REAL *w_in, const REAL *b_in, const REAL *mid, REAL *dist, int *idx)
{
    int k;
    for (k = 0; k < all; ++k) {
        const REAL *w = w_in + 3 * k;
        REAL acc = w[0] * mid[0] + w[1] * mid[1] + w[2] * mid[2] + b_in[k];
        dist[k] = acc * FN(rsq)(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        idx[k] = k;
    }
    /* insertion-merge: simple stable merge sort */
    {
        int width;
        int *tmp = (int *)malloc(sizeof(int) * (size_t)all);
        for (width = 1; width < all; width *= 2) {
            int lo;
            for (lo = 0; lo < all; lo += 2 * width) {
                int mid_ = lo + width < all ? lo + width : all;
                int hi = lo + 2 * width < all ? lo + 2 * width : all;
                int a = lo, b = mid_, o = lo;
                while (a < mid_ && b < hi) {
                    REAL da = dist[idx[a]], db = dist[idx[b]];
                    /* take b first only if db > da (strict), NaN last */
                    int take_b;
                    if (da != da) take_b = (db == db);
                    else if (db != db) take_b = 0;
                    else take_b = db > da;
                    tmp[o++] = take_b ? idx[b++] : idx[a++];
                }
                while (a < mid_) tmp[o++] = idx[a++];
                while (b < hi) tmp[o++] = idx[b++];
            }
            memcpy(idx, tmp, sizeof(int) * (size_t)all);
        }
        free(tmp);
    }
}

/* cudaCheckCondition_kernel / cudaCheckCondition2_kernel feasibility test,
 * kernel.h:729-795 and kernel.h:1024-1097 (geometric distance, macro.h:6). */
static int FN(feasible)(int all, const REAL *w_in, const REAL *b_in, const REAL *x, int ei, int ej)
{
    int k;
    for (k = 0; k < all; ++k) {
        const REAL *w = w_in + 3 * k;
        REAL ans = w[0] * x[0] + w[1] * x[1] + w[2] * x[2] + b_in[k];
        REAL rs = FN(rsq)(w[0] * w[0] + w[1] * w[1] + w[2] * w[2]);
        if (ans * rs > R_EPS && k != ei && k != ej) return 0;
    }
    return 1;
}

static void FN(make_sys)(const REAL *w_in, const REAL *b_in, const REAL *w_eq, REAL b_eq, int r1, int r2, REAL *A, REAL *bb)
{
    A[0] = w_in[3 * r1 + 0]; A[1] = w_in[3 * r1 + 1]; A[2] = w_in[3 * r1 + 2];
    A[3] = w_in[3 * r2 + 0]; A[4] = w_in[3 * r2 + 1]; A[5] = w_in[3 * r2 + 2];
    A[6] = w_eq[0]; A[7] = w_eq[1]; A[8] = w_eq[2];
    bb[0] = b_in[r1]; bb[1] = b_in[r2]; bb[2] = b_eq;
}

/* existInArray, kernel.h:882-896 */
static int FN(exist)(const int *entries, int query, int n)
{
    int k;
    for (k = 0; k < n; ++k) {
        int t = entries[k];
        t = t >= 0 ? t : (-t - 1);
        if (t == query) return 1;
    }
    return 0;
}

/* isPivotValid_ / isPivotValid, kernel.h:1103-1149 */
static int FN(pivot_valid)(const REAL *neq, const REAL *w_in, const int *tab, int new_i, int *last_idx)
{
    int tab_idx = tab[0], cnt = 0, ref_idx = 1;
    while (tab_idx >= 1 && cnt < 2) {
        if (tab[tab_idx] >= 0) {
            if (cnt == 0) { *last_idx = tab_idx; cnt++; }
            else if (cnt == 1) { ref_idx = tab_idx; cnt++; }
        }
        tab_idx--;
    }
    if (cnt != 2) return -1;
    {
        const REAL *n1 = w_in + 3 * tab[ref_idx];
        const REAL *n2 = w_in + 3 * tab[*last_idx];
        const REAL *n3 = w_in + 3 * new_i;
#define AMO_DOT(a, b) ((a)[0] * (b)[0] + (a)[1] * (b)[1] + (a)[2] * (b)[2])
        REAL A12 = AMO_DOT(n1, n2), A23 = AMO_DOT(n2, n3), A13 = AMO_DOT(n1, n3), A22 = AMO_DOT(n2, n2);
        REAL C1 = AMO_DOT(n1, neq), C2 = AMO_DOT(n2, neq), C3 = AMO_DOT(n3, neq), B = AMO_DOT(neq, neq);
#undef AMO_DOT
        return ((A12 * A23 - A22 * A13) - (A12 * C2 * C3 + A23 * C1 * C2 - A13 * C2 * C2 - A22 * C1 * C3) / B) > 0;
    }
}

/* One 3x3 system of a round: the rows of cnt_x2 (state, a, b, c, ok). */
typedef struct {
    int st, x, ri, rj, ok;
} FN(amo_sys);

/* Per-batch region data kept for the round simulation. */
typedef struct {
    int bsz, all, N;
    REAL *w_in, *b_in, *weq; /* bsz x all x 3, bsz x all, bsz x 4 */
    int *idx;                /* bsz x all, distance order */
    int *start;              /* bsz, FACEDATA.start_idx */
    REAL *vert;              /* bsz x (1 + 3 VM), vertices_buffer */
    int *tab;                /* bsz x (2 + VM), tabij */
} FN(amo_batch);

static void FN(solve_check)(const FN(amo_batch) *bt, FN(amo_sys) *sys, REAL *xs, int nsys)
{
    int s;
#pragma omp parallel for schedule(dynamic, 16)
    for (s = 0; s < nsys; ++s) {
        const int st = sys[s].st;
        const REAL *w_in = bt->w_in + (size_t)st * bt->all * 3;
        const REAL *b_in = bt->b_in + (size_t)st * bt->all;
        const REAL *weq = bt->weq + 4 * (size_t)st;
        REAL A[9], bb[3];
        FN(make_sys)(w_in, b_in, weq, weq[3], sys[s].ri, sys[s].rj, A, bb);
        FN(solve3)(A, bb, xs + 3 * s);
        if (!FN(feasible)(bt->all, w_in, b_in, xs + 3 * s, sys[s].ri, sys[s].rj)) sys[s].ok = 0;
    }
}

/* calcStartIdx, kernel.h:799-856, as SOLVE_SIZE_MAX threads per round in
 * thread-index order: cudaInitCntX (kernel.cu:172-197), fillAs_kernel
 * (kernel.h:626-705, pairs from get_i_j), solve_3x3, cudaCheckCondition
 * (kernel.h:729-795), cudaUpdateStartIdx (kernel.cu:80-101: the last ok
 * system of a round wins), cudaInitCntX2 (kernel.cu:105-167). */
static void FN(start_rounds)(FN(amo_batch) *bt, FN(amo_sys) *sys, REAL *xs, int *cs_state, int *cs_x, int *xbs)
{
    const int bsz = bt->bsz, all = bt->all;
    int x_max = (all - 1) * (all - 2), num = 0, tid;
    if (x_max > 812) x_max = 812;
    for (tid = 0; tid < bsz; ++tid)
        if (bt->start[tid] == -1) { cs_state[num] = tid; cs_x[num] = 0; num++; }
    while (num > 0) {
        int nsys = 0, s;
        for (tid = 0; tid < AMO_SOLVE_MAX; ++tid) {
            int mod = tid % num, st = cs_state[mod], x = cs_x[mod] + tid / num;
            if (x <= x_max) {
                int i, j;
                amo_get_i_j(x, all, &i, &j);
                sys[nsys].st = st;
                sys[nsys].x = x;
                sys[nsys].ri = bt->idx[(size_t)st * all + i];
                sys[nsys].rj = bt->idx[(size_t)st * all + j];
                sys[nsys].ok = 1;
                nsys++;
            }
        }
        FN(solve_check)(bt, sys, xs, nsys);
        for (s = 0; s < nsys; ++s)
            if (sys[s].ok) bt->start[sys[s].st] = sys[s].ri;
        for (tid = 0; tid < bsz; ++tid) xbs[tid] = -1;
        for (s = 0; s < nsys; ++s)
            if (sys[s].x > xbs[sys[s].st]) xbs[sys[s].st] = sys[s].x;
        for (s = 0; s < nsys; ++s)
            if (sys[s].ok || sys[s].x > x_max) xbs[sys[s].st] = -1;
        num = 0;
        for (tid = 0; tid < bsz; ++tid)
            if (xbs[tid] != -1) { cs_state[num] = tid; cs_x[num] = xbs[tid] + 1; num++; }
    }
}

/* calcPivoting, kernel.h:1258-1320, as SOLVE_SIZE_MAX threads per round in
 * thread-index order: cudaInitCntX3 (kernel.h:861-899), fillAs2_kernel
 * (kernel.h:903-998, per-region candidate cursor), solve_3x3,
 * cudaCheckCondition2 (kernel.h:1024-1097), cudaUpdateVert_kernel
 * (kernel.h:1157-1230: the first ok system takes the region's mutex), and
 * cudaInitCntX4 (kernel.cu:203-299).  vert / tab have exactly the layout of
 * vertices_buffer / tabij. */
static void FN(pivot_rounds)(FN(amo_batch) *bt, FN(amo_sys) *sys, REAL *xs, int *cp_state, int *cp_start, int *cp_wrap,
                             int *offset, int *bs1, int *bs2, int *bs3, int *bs4, int *mutex)
{
    const int bsz = bt->bsz, all = bt->all, VM = AMO_VERT_MAX;
    int num = 0, tid;
    for (tid = 0; tid < bsz; ++tid) {
        int *tab = bt->tab + (size_t)tid * (2 + VM);
        REAL *vert = bt->vert + (size_t)tid * (1 + 3 * VM);
        tab[0] = 0;
        vert[0] = 0;
        if (bt->start[tid] != -1) {
            cp_state[num] = tid;
            cp_start[num] = bt->start[tid];
            cp_wrap[num] = 0;
            num++;
            tab[0] = 1;
            tab[1] = bt->start[tid];
        }
    }
    while (num > 0) {
        int nsys = 0, s;
        for (tid = 0; tid < bsz; ++tid) offset[tid] = 0;
        for (tid = 0; tid < AMO_SOLVE_MAX; ++tid) {
            const int mod = tid % num, st = cp_state[mod];
            const int *tab = bt->tab + (size_t)st * (2 + VM);
            for (;;) {
                int wrap_i = cp_wrap[mod] + offset[st]++;
                int real_i;
                if (wrap_i >= all) break;
                real_i = bt->idx[(size_t)st * all + wrap_i];
                if ((real_i == tab[1] && tab[0] >= 3) || !FN(exist)(tab + 1, real_i, tab[0])) {
                    sys[nsys].st = st;
                    sys[nsys].ri = real_i;      /* row 1 of the system */
                    sys[nsys].rj = cp_start[mod]; /* row 2: current edge plane */
                    sys[nsys].x = wrap_i;
                    sys[nsys].ok = 1;
                    nsys++;
                    break;
                }
            }
        }
        FN(solve_check)(bt, sys, xs, nsys);
        for (tid = 0; tid < bsz; ++tid) { bs1[tid] = -1; bs2[tid] = -1; mutex[tid] = -1; }
        for (s = 0; s < nsys; ++s) {
            const int st = sys[s].st, new_i = sys[s].ri;
            int *tab = bt->tab + (size_t)st * (2 + VM);
            REAL *vert = bt->vert + (size_t)st * (1 + 3 * VM);
            const REAL *weq = bt->weq + 4 * (size_t)st;
            const REAL *w_in = bt->w_in + (size_t)st * all * 3;
            const REAL *x = xs + 3 * s;
            int close = ((tab[0] >= 4 && tab[1] == tab[tab[0]]) || tab[0] >= VM + 1);
            int last_idx = 1, start_index, pv;
            if (!(sys[s].ok && !close)) continue;
            if (mutex[st] != -1) continue;
            mutex[st] = s;
            pv = FN(pivot_valid)(weq, w_in, tab, new_i, &last_idx);
            if (pv == 0) {
                tab[++tab[0]] = -new_i - 1;
                start_index = last_idx; /* kernel.h:1189 keeps the tab position, not the plane */
            } else {
                int nv = (int)vert[0];
                const REAL *lv = vert + (3 * nv - 2);
                /* isSameVertices, kernel.h:1151-1155 */
                if (nv > 0 && (CAT(amo_fabs, SFX)(lv[0] - x[0]) + CAT(amo_fabs, SFX)(lv[1] - x[1]) +
                               CAT(amo_fabs, SFX)(lv[2] - x[2])) < R_SAME_EPS) {
                    tab[++tab[0]] = new_i;
                    start_index = new_i;
                    tab[last_idx] = -tab[last_idx] - 1;
                } else {
                    int o = 3 * nv + 1;
                    vert[o + 0] = x[0];
                    vert[o + 1] = x[1];
                    vert[o + 2] = x[2];
                    vert[0] = (REAL)(nv + 1);
                    tab[++tab[0]] = new_i;
                    start_index = new_i;
                }
            }
            if ((tab[0] >= 4 && tab[1] == tab[tab[0]]) || tab[0] >= VM + 1) { bs1[st] = -2; bs2[st] = -2; }
            else { bs1[st] = start_index; bs2[st] = 0; }
        }
        for (tid = 0; tid < bsz; ++tid) { bs3[tid] = -1; bs4[tid] = -1; }
        for (s = 0; s < nsys; ++s) {
            bs3[sys[s].st] = sys[s].rj;
            if (sys[s].x > bs4[sys[s].st]) bs4[sys[s].st] = sys[s].x;
        }
        for (tid = 0; tid < bsz; ++tid) {
            if (bs3[tid] == -1) continue;
            if (bs1[tid] >= 0 && bs2[tid] >= 0) { bs3[tid] = bs1[tid]; bs4[tid] = bs2[tid]; }
            else if (bs1[tid] == -1 && bs2[tid] == -1) {
                bs4[tid]++;
                if (bs4[tid] >= all) { bs3[tid] = -1; bs4[tid] = -1; } /* "we cannot find solution" */
            } else if (bs1[tid] == -2 && bs2[tid] == -2) { bs3[tid] = -1; bs4[tid] = -1; }
        }
        num = 0;
        for (tid = 0; tid < bsz; ++tid)
            if (bs3[tid] != -1 && bs4[tid] != -1) { cp_state[num] = tid; cp_start[num] = bs3[tid]; cp_wrap[num] = bs4[tid]; num++; }
    }
}

/* correctNormalDirection_kernel, kernel.h:1325-1370 */
static void FN(orient)(REAL *vert, const REAL *w_eq, int flip)
{
    int num = (int)vert[0];
    if (num >= 3) {
        REAL ax = vert[4] - vert[1], ay = vert[5] - vert[2], az = vert[6] - vert[3];
        REAL bx = vert[7] - vert[4], by = vert[8] - vert[5], bz = vert[9] - vert[6];
        REAL cx = ay * bz - az * by, cy = az * bx - ax * bz, cz = ax * by - ay * bx;
        REAL dir = cx * w_eq[0] + cy * w_eq[1] + cz * w_eq[2];
        if ((dir < 0) ^ (flip != 0)) {
            int h = num / 2, q;
            for (q = 0; q < h; ++q) {
                int a = 3 * q + 1, b = 3 * (num - q) - 2, c;
                for (c = 0; c < 3; ++c) {
                    REAL t = vert[a + c];
                    vert[a + c] = vert[b + c];
                    vert[b + c] = t;
                }
            }
        }
    }
}

typedef struct {
    uint32_t *bits;    /* cap x words */
    REAL *mid;         /* cap x 3 */
    int *start;        /* cap */
    long cap, num;
} FN(amo_stack);

static void FN(stack_reserve)(FN(amo_stack) *s, long need, int words)
{
    if (need <= s->cap) return;
    {
        long nc = s->cap ? s->cap : 1024;
        while (nc < need) nc *= 2;
        s->bits = (uint32_t *)realloc(s->bits, sizeof(uint32_t) * (size_t)nc * (size_t)words);
        s->mid = (REAL *)realloc(s->mid, sizeof(REAL) * 3 * (size_t)nc);
        s->start = (int *)realloc(s->start, sizeof(int) * (size_t)nc);
        s->cap = nc;
    }
}

/* encode (hash.h:15-31): byte j bit k = state[8j + k] -- with packed uint32
 * words in little-endian order the byte string is the word array itself. */
static void FN(encode)(const uint32_t *bits, int N, uint8_t *out)
{
    int nb = (N + 7) / 8, q;
    for (q = 0; q < nb; ++q) out[q] = (uint8_t)((bits[q >> 2] >> (8 * (q & 3))) & 0xffu);
}

/* try_insert, hash.h:33-67 (device path: CAS on HASH2_ZERO) */
static int FN(try_insert)(uint32_t *table, uint32_t mask, uint32_t zero, const uint8_t *bytes, int nb)
{
    uint32_t idx = amo_fnv1a(bytes, nb) & mask;
    uint32_t value = amo_fnv1(bytes, nb);
    for (;;) {
        uint32_t prev = table[idx];
        if (prev == zero) { table[idx] = value; return 1; }
        if (prev == value) return 0;
        idx = (idx + 1543u) & mask;
    }
}

static int FN(run)(const amo_net *net, const uint8_t *states, const REAL *points, int S, double iso_d, int flip,
                   amo_result **out)
{
    FN(amo_view) v;
    amo_result *res;
    int N = 0, words, nb, i;
    const uint32_t TABLE_SIZE = 33554432u; /* macro.h:34 _STATES_TABLE_SIZE */
    uint32_t *table;
    uint32_t zero;
    uint8_t *tmpb;
    FN(amo_stack) st;
    const REAL iso = (REAL)iso_d;

    memset(&v, 0, sizeof(v));
    v.net = net;
    if (net->n_lin < 2 || net->n_lin > 62 || net->nodes[0] != 3 || net->nodes[net->n_lin] != 1) return -1;
    v.offs[0] = 0;
    for (i = 1; i <= net->n_lin; ++i) v.offs[i] = v.offs[i - 1] + net->nodes[i];
    for (i = 1; i < net->n_lin; ++i) N += net->nodes[i];
    v.maxw = 0;
    for (i = 0; i <= net->n_lin; ++i) v.maxw = net->nodes[i] > v.maxw ? net->nodes[i] : v.maxw;
    v.N = N;
    v.E = net->E;
    v.all = N + net->E;
    words = (N + 31) / 32;
    nb = (N + 7) / 8;

    res = (amo_result *)calloc(1, sizeof(amo_result));
    res->N = N;
    res->words = words;
    res->is_f64 = (sizeof(REAL) == 8);

    table = (uint32_t *)malloc(sizeof(uint32_t) * TABLE_SIZE);
    tmpb = (uint8_t *)calloc((size_t)nb + 8, 1);
    zero = amo_fnv1(tmpb, nb); /* get_hash2_zero, states.h:209-216 */
    {
        uint32_t q;
        for (q = 0; q < TABLE_SIZE; ++q) table[q] = zero;
    }

    /* STATES::reinit, states.h:147-176: hash-dedup seeds, keep survivors in order */
    memset(&st, 0, sizeof(st));
    FN(stack_reserve)(&st, S > 0 ? S : 1, words);
    {
        uint32_t *pk = (uint32_t *)calloc((size_t)words, sizeof(uint32_t));
        int s;
        for (s = 0; s < S; ++s) {
            int k;
            memset(pk, 0, sizeof(uint32_t) * (size_t)words);
            for (k = 0; k < N; ++k)
                if (states[(size_t)s * N + k]) pk[k >> 5] |= 1u << (k & 31);
            FN(encode)(pk, N, tmpb);
            if (FN(try_insert)(table, TABLE_SIZE - 1, zero, tmpb, nb)) {
                memcpy(st.bits + (size_t)st.num * words, pk, sizeof(uint32_t) * (size_t)words);
                st.mid[3 * st.num + 0] = points[3 * s + 0];
                st.mid[3 * st.num + 1] = points[3 * s + 1];
                st.mid[3 * st.num + 2] = points[3 * s + 2];
                st.start[st.num] = -1;
                st.num++;
            }
        }
        free(pk);
    }
    res->seeds_kept = (int)st.num;

    /* main_ loop, cuam_kernel.cu:53-97 */
    {
        const int all = v.all;
        const int VM = AMO_VERT_MAX;
        const int B = AMO_BATCH_MAX;
        uint32_t *bb_bits = (uint32_t *)malloc(sizeof(uint32_t) * B * (size_t)words);
        REAL *bb_mid = (REAL *)malloc(sizeof(REAL) * 3 * B);
        FN(amo_batch) bt;
        FN(amo_sys) *sys = (FN(amo_sys) *)malloc(sizeof(FN(amo_sys)) * AMO_SOLVE_MAX);
        REAL *xs = (REAL *)malloc(sizeof(REAL) * 3 * AMO_SOLVE_MAX);
        int *ib = (int *)malloc(sizeof(int) * 11 * (size_t)B);
        uint32_t *child = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)words);
        bt.all = all;
        bt.N = N;
        bt.w_in = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)B * all);
        bt.b_in = (REAL *)malloc(sizeof(REAL) * (size_t)B * all);
        bt.weq = (REAL *)malloc(sizeof(REAL) * 4 * B);
        bt.idx = (int *)malloc(sizeof(int) * (size_t)B * all);
        bt.start = (int *)malloc(sizeof(int) * B);
        bt.vert = (REAL *)malloc(sizeof(REAL) * (1 + 3 * VM) * B);
        bt.tab = (int *)malloc(sizeof(int) * (2 + VM) * B);

        while (st.num > 0) {
            int bsz = st.num < B ? (int)st.num : B;
            int b;
            st.num -= bsz; /* STATES::pop_back, states.h:220-243 */
            memcpy(bb_bits, st.bits + (size_t)st.num * words, sizeof(uint32_t) * (size_t)bsz * words);
            memcpy(bb_mid, st.mid + 3 * st.num, sizeof(REAL) * 3 * (size_t)bsz);
            memcpy(bt.start, st.start + st.num, sizeof(int) * (size_t)bsz);
            bt.bsz = bsz;

            /* fill_constraints, offset_b_equ, fill_distance, sortDistance */
#pragma omp parallel
            {
                REAL *dist = (REAL *)malloc(sizeof(REAL) * (size_t)all);
                REAL *wt = (REAL *)malloc(sizeof(REAL) * 3 * (size_t)(v.maxw + 1));
                REAL *btmp = (REAL *)malloc(sizeof(REAL) * (size_t)(v.maxw + 1));
#pragma omp for schedule(dynamic, 8)
                for (b = 0; b < bsz; ++b) {
                    REAL *w_in = bt.w_in + (size_t)b * all * 3;
                    REAL *b_in = bt.b_in + (size_t)b * all;
                    REAL *weq = bt.weq + 4 * b;
                    FN(compose)(&v, bb_bits + (size_t)b * words, iso, w_in, b_in, weq, weq + 3, wt, btmp);
                    FN(sort_dist)(all, w_in, b_in, bb_mid + 3 * b, dist, bt.idx + (size_t)b * all);
                }
                free(dist); free(wt); free(btmp);
            }
            /* fillStartIdx (seeds only) and vertPivoting */
            {
                int any = 0;
                for (b = 0; b < bsz; ++b) any |= (bt.start[b] == -1); /* cudaCheckAnyEqual, kernel.h:799-804 */
                if (any) FN(start_rounds)(&bt, sys, xs, ib, ib + B, ib + 2 * B);
            }
            FN(pivot_rounds)(&bt, sys, xs, ib, ib + B, ib + 2 * B, ib + 3 * B, ib + 4 * B, ib + 5 * B, ib + 6 * B,
                             ib + 7 * B, ib + 8 * B);
            /* corrNormDir */
            for (b = 0; b < bsz; ++b) FN(orient)(bt.vert + (size_t)b * (1 + 3 * VM), bt.weq + 4 * b, flip);

            /* record the batch (one record per popped state) */
            {
                long need = res->num + bsz;
                if (need > res->cap) {
                    long nc = res->cap ? res->cap : 4096;
                    while (nc < need) nc *= 2;
                    res->bits = (uint32_t *)realloc(res->bits, sizeof(uint32_t) * (size_t)nc * words);
                    res->nverts = (int *)realloc(res->nverts, sizeof(int) * (size_t)nc);
                    res->verts = (double *)realloc(res->verts, sizeof(double) * (size_t)nc * VM * 3);
                    res->ntab = (int *)realloc(res->ntab, sizeof(int) * (size_t)nc);
                    res->tab = (int *)realloc(res->tab, sizeof(int) * (size_t)nc * (VM + 1));
                    res->mid = (double *)realloc(res->mid, sizeof(double) * (size_t)nc * 3);
                    res->start = (int *)realloc(res->start, sizeof(int) * (size_t)nc);
                    res->cap = nc;
                }
                for (b = 0; b < bsz; ++b) {
                    long r = res->num + b;
                    const REAL *vt = bt.vert + (size_t)b * (1 + 3 * VM);
                    const int *tb = bt.tab + (size_t)b * (2 + VM);
                    int q;
                    memcpy(res->bits + (size_t)r * words, bb_bits + (size_t)b * words, sizeof(uint32_t) * (size_t)words);
                    res->nverts[r] = (int)vt[0];
                    for (q = 0; q < 3 * VM; ++q) res->verts[(size_t)r * VM * 3 + q] = (double)vt[1 + q];
                    res->ntab[r] = tb[0];
                    for (q = 0; q < VM + 1; ++q) res->tab[(size_t)r * (VM + 1) + q] = tb[1 + q];
                    for (q = 0; q < 3; ++q) res->mid[(size_t)r * 3 + q] = (double)bb_mid[3 * b + q];
                    res->start[r] = bt.start[b];
                }
                res->num += bsz;
            }

            /* inferNewStates_kernel (kernel.h:1390-1478) in thread-index order
             * (tid = vert_idx * batch + batch_idx), then STATES::push_back */
            {
                int vi;
                for (vi = 0; vi < VM; ++vi) {
                    for (b = 0; b < bsz; ++b) {
                        const int *tab = bt.tab + (size_t)b * (2 + VM) + 1; /* tab[-1] = count */
                        const REAL *vert = bt.vert + (size_t)b * (1 + 3 * VM) + 1;
                        int tabij_num = tab[-1];
                        int switch_i;
                        if (!(vi < tabij_num - 1)) continue;
                        switch_i = tab[vi];
                        if (!(switch_i >= 0 && switch_i < N)) continue;
                        memcpy(child, bb_bits + (size_t)b * words, sizeof(uint32_t) * (size_t)words);
                        child[switch_i >> 5] ^= 1u << (switch_i & 31);
                        FN(encode)(child, N, tmpb);
                        if (FN(try_insert)(table, TABLE_SIZE - 1, zero, tmpb, nb)) {
                            int cnt_idx = -1, v1 = 0, v2, q;
                            int vi_ = (vi == 0) ? (tabij_num - 1) : vi;
                            int nvv = (int)vert[-1];
                            for (q = 1; q < tabij_num; ++q) {
                                if (tab[q] >= 0) cnt_idx++;
                                if (q == vi_) v1 = cnt_idx;
                            }
                            if (v1 < 0) v1 = 0;   /* unreachable for well-formed tabs */
                            v2 = nvv > 0 ? (v1 + 1) % nvv : 0;
                            FN(stack_reserve)(&st, st.num + 1, words);
                            memcpy(st.bits + (size_t)st.num * words, child, sizeof(uint32_t) * (size_t)words);
                            for (q = 0; q < 3; ++q) st.mid[3 * st.num + q] = (vert[3 * v1 + q] + vert[3 * v2 + q]) / 2;
                            st.start[st.num] = switch_i;
                            st.num++;
                        }
                    }
                }
            }
            if (g_region_budget > 0 && res->num >= g_region_budget) break;
        }
        free(bb_bits); free(bb_mid); free(sys); free(xs); free(ib); free(child);
        free(bt.w_in); free(bt.b_in); free(bt.weq); free(bt.idx); free(bt.start); free(bt.vert); free(bt.tab);
    }

    free(table);
    free(tmpb);
    free(st.bits); free(st.mid); free(st.start);
    *out = res;
    return 0;
}

/* PointHash1 / PointHash2 over the 12 bytes of three int32, polymesh.h:144-170 */
static void FN(point_key)(const double *p, int *key)
{
    REAL x = (REAL)p[0], y = (REAL)p[1], z = (REAL)p[2];
    key[0] = (int)(x * (REAL)R_PH_MUL);
    key[1] = (int)(y * (REAL)R_PH_MUL);
    key[2] = (int)(z * (REAL)R_PH_MUL);
}

/* PolyMesh::combine_mesh, polymesh.h:339-346: uniqueVertHash (174-233),
 * indexingVertices (237-264), indexingFaces (268-335); processed in
 * polygon order (the reference assigns indices with atomicAdd). */
static int FN(combine)(amo_result *r, double scale, const double *center)
{
    const uint32_t HASH_LEN = 33554432u, MASK = HASH_LEN - 1u, SKIP = 1543u;
    const int VM = AMO_VERT_MAX;
    int *hash = (int *)malloc(sizeof(int) * 2 * (size_t)HASH_LEN);
    long p, nv = 0, nf = 0;
    long *offs;
    uint32_t q;
    for (q = 0; q < 2 * HASH_LEN; ++q) hash[q] = -1;
    offs = (long *)malloc(sizeof(long) * ((size_t)r->num * VM + 1));
    for (p = 0; p < r->num; ++p) {
        int i, num = r->nverts[p];
        for (i = 0; i < num; ++i) {
            int key[3];
            uint32_t idx;
            int value;
            FN(point_key)(r->verts + ((size_t)p * VM + i) * 3, key);
            idx = amo_fnv1a((const uint8_t *)key, 12) & MASK;
            value = (int)amo_fnv1((const uint8_t *)key, 12);
            for (;;) {
                int prev = hash[2 * idx + 1];
                if (prev == -1) hash[2 * idx + 1] = value;
                if (prev == value) break;
                if (prev == -1) {
                    hash[2 * idx] = (int)nv;
                    offs[nv] = (long)(p * VM + i);
                    nv++;
                    break;
                }
                idx = (idx + SKIP) & MASK;
            }
        }
    }
    free(r->mverts);
    free(r->mfaces);
    r->mverts = (double *)malloc(sizeof(double) * 3 * (size_t)(nv + 1));
    {
        long t;
        for (t = 0; t < nv; ++t) {
            int c;
            for (c = 0; c < 3; ++c) {
                REAL val = (REAL)r->verts[offs[t] * 3 + c] * (REAL)scale + (REAL)center[c];
                r->mverts[3 * t + c] = (double)val;
            }
        }
    }
    r->mfaces = (int *)malloc(sizeof(int) * (1 + VM) * ((size_t)r->num + 1));
    for (p = 0; p < r->num; ++p) {
        int i, num = r->nverts[p];
        if (num < 3) continue;
        r->mfaces[(size_t)nf * (1 + VM)] = num;
        for (i = 0; i < num; ++i) {
            int key[3];
            uint32_t idx;
            int value, vi = -1;
            FN(point_key)(r->verts + ((size_t)p * VM + i) * 3, key);
            idx = amo_fnv1a((const uint8_t *)key, 12) & MASK;
            value = (int)amo_fnv1((const uint8_t *)key, 12);
            for (;;) {
                if (hash[2 * idx + 1] == value) { vi = hash[2 * idx]; break; }
                idx = (idx + SKIP) & MASK;
            }
            r->mfaces[(size_t)nf * (1 + VM) + 1 + i] = vi;
        }
        nf++;
    }
    r->mesh_nv = (int)nv;
    r->mesh_nf = (int)nf;
    free(offs);
    free(hash);
    return 0;
}

#undef FN
#undef CAT
#undef CAT_
