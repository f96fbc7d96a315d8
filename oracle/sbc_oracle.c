/*
 * Parity oracle for the StreamingBC hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file is a plain-C restatement of the reference's COARSE CPU path:
 * the static Brandes init and the per-root incremental update that runs on
 * every edge insertion.  It exists to check the CUDA path and to time the
 * reference algorithm on the host (the "port" CPU baseline).  Nothing in the
 * product library links or calls it; only the tests, the smoke check and the
 * CPU-baseline leg of the benchmark load it.
 *
 * Reference files followed (paths inside the ogreen/StreamingBC tree):
 *   static init      src/streamingbc_init.c:60-84   (BrandesApproxCaseParallel)
 *                    src/streamingbc_init.c:87-183  (BrandesSingleTree)
 *   dispatcher       src/streamingbc.c:88-226       (insertEdgeStreamingBC, COARSE)
 *   |d| == 1         src/streamingbc_internal.c:11-248   (addEdgeWithoutMovementBrandes)
 *   |d|  > 1         src/streamingbc_internal.c:251-603  (moveUpTreeBrandes)
 *   level buckets    src/streamingbc_aux.c:372-427  (appendDS / getFirstDS / deleteFirstDS)
 *   scratch init     src/streamingbc_aux.c:234-296  (createExtraArraysPerThread)
 *
 * Deliberate differences, none of which changes level, sigma, delta or BC:
 *   - State is structure-of-arrays [root][vertex] instead of the 40-byte bcV
 *     record, and edgesAbove / edgesBelow are not carried (they only feed the
 *     BALANCE ordering heuristic, src/streamingbc.c:104-122).
 *   - Roots are visited in root-array order (NO_BALANCE order).  Results do not
 *     depend on the visiting order beyond floating-point summation order.
 *   - The |d| > 1 descent computes a neighbour's movement from the current
 *     vertex's NEW level (c = level[k] - newLevel[cur] - 1).  This is the same
 *     integer as the reference's movementDelta - (level[cur]-level[k]+1), but it
 *     never overflows when a level is "infinite" (LONG_MAX), where the reference
 *     relies on wrapping signed arithmetic.
 *   - The stale-entry read of the Up queue in the |d| == 1 ascent merge
 *     (src/streamingbc_internal.c:144-149) is replaced by a bounds-checked
 *     merge; the reference never reaches the stale entry on valid input.
 *
 * Everything else -- unreachable level/sigma = INT64_MAX, BC as the raw sum of
 * delta over roots excluding the root itself, per-thread BC partials reduced
 * after every call, the O(NV) level-bucket drain of the |d| > 1 path, and the
 * traversal counters -- follows the reference.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#define ORC_INF INT64_MAX

/* ------------------------------------------------------------------------ */
/* Graph: per-vertex growable neighbour arrays (stands in for STINGER).      */
/* ------------------------------------------------------------------------ */

typedef struct {
    int64_t nv;
    int64_t *deg;
    int64_t *cap;
    int64_t **nbr;
} orc_graph;

orc_graph *orc_graph_new(int64_t nv, const int64_t *off, const int64_t *adj)
{
    orc_graph *g = (orc_graph *)calloc(1, sizeof(orc_graph));
    if (!g) return NULL;
    g->nv = nv;
    g->deg = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    g->cap = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    g->nbr = (int64_t **)calloc((size_t)nv, sizeof(int64_t *));
    for (int64_t v = 0; v < nv; v++) {
        int64_t d = off[v + 1] - off[v];
        int64_t c = d < 4 ? 4 : d + d / 4;
        g->nbr[v] = (int64_t *)malloc((size_t)c * sizeof(int64_t));
        g->cap[v] = c;
        g->deg[v] = d;
        if (d) memcpy(g->nbr[v], adj + off[v], (size_t)d * sizeof(int64_t));
    }
    return g;
}

void orc_graph_free(orc_graph *g)
{
    if (!g) return;
    for (int64_t v = 0; v < g->nv; v++) free(g->nbr[v]);
    free(g->nbr); free(g->deg); free(g->cap); free(g);
}

int64_t orc_graph_degree(const orc_graph *g, int64_t v) { return g->deg[v]; }

/* Directed insert with the return convention of stinger_insert_edge
 * (src/stinger/stinger.c:778-876): -1 self loop, 0 already present, 1 new. */
/* Remove `to` from the neighbours of `from` (stinger_remove_edge,
 * src/stinger/stinger.c): 1 removed, 0 absent.  Order of the remaining
 * neighbours is kept. */
int orc_graph_remove(orc_graph *g, int64_t from, int64_t to)
{
    for (int64_t i = 0; i < g->deg[from]; i++) {
        if (g->nbr[from][i] != to) continue;
        for (int64_t j = i + 1; j < g->deg[from]; j++) g->nbr[from][j - 1] = g->nbr[from][j];
        g->deg[from]--;
        return 1;
    }
    return 0;
}

int orc_graph_insert(orc_graph *g, int64_t from, int64_t to)
{
    if (from == to) return -1;
    for (int64_t i = 0; i < g->deg[from]; i++)
        if (g->nbr[from][i] == to) return 0;
    if (g->deg[from] == g->cap[from]) {
        int64_t c = g->cap[from] * 2;
        int64_t *p = (int64_t *)realloc(g->nbr[from], (size_t)c * sizeof(int64_t));
        if (!p) return -1;
        g->nbr[from] = p;
        g->cap[from] = c;
    }
    g->nbr[from][g->deg[from]++] = to;
    return 1;
}

/* ------------------------------------------------------------------------ */
/* Forest and per-thread scratch.                                            */
/* ------------------------------------------------------------------------ */

typedef struct {
    /* per-vertex scratch, restating sbcV (src/streamingbc_aux.h:130-144) */
    int64_t *diff;     /* diffPath */
    int64_t *touched;
    int64_t *nsig;     /* newSigma */
    int64_t *nlev;     /* new level of a descent vertex (|d| > 1) */
    int64_t *moved;    /* IMoved: -1 untouched, 0 kept its level, 1 moved up */
    double *ndelta;    /* newDelta */
    double *bcpart;    /* per-thread BC partial (sV[].totalBC) */
    int64_t *qdown, *qup, *qsame;
    /* level buckets (queue_t + level_node_t, src/streamingbc_aux.c:372-427) */
    int64_t *bfront, *bback, *bnext, *bdata;
    int64_t bsize;
    /* traversal counters (COUNT_TRAVERSALS, src/streamingbc_aux.h:12) */
    int64_t tv, te, n1, n2;
} orc_scratch;

typedef struct {
    int64_t nv, nk, nt;
    int64_t nt_active; /* threads the parallel loops use (<= nt; the reference's NT) */
    int64_t *roots;
    int64_t *level;   /* [nk][nv] */
    int64_t *sigma;   /* [nk][nv] */
    double *delta;    /* [nk][nv] */
    double *bc;       /* [nv] */
    orc_scratch *scr; /* [nt] */
    /* counters of the last static / insert call, summed over threads */
    int64_t last_tv, last_te, last_case1, last_case2;
} orc_forest;

static void scratch_init(orc_scratch *s, int64_t nv)
{
    memset(s, 0, sizeof(*s));
    s->diff = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    s->touched = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    s->nsig = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    s->nlev = (int64_t *)calloc((size_t)nv, sizeof(int64_t));
    s->moved = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->ndelta = (double *)calloc((size_t)nv, sizeof(double));
    s->bcpart = (double *)calloc((size_t)nv, sizeof(double));
    s->qdown = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->qup = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->qsame = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->bfront = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->bback = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->bnext = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    s->bdata = (int64_t *)malloc((size_t)nv * sizeof(int64_t));
    for (int64_t v = 0; v < nv; v++) {
        s->moved[v] = -1;
        s->bfront[v] = -1;
        s->bback[v] = -1;
    }
}

static void scratch_free(orc_scratch *s)
{
    free(s->diff); free(s->touched); free(s->nsig); free(s->nlev); free(s->moved);
    free(s->ndelta); free(s->bcpart); free(s->qdown); free(s->qup); free(s->qsame);
    free(s->bfront); free(s->bback); free(s->bnext); free(s->bdata);
}

orc_forest *orc_forest_new(int64_t nv, int64_t nk, const int64_t *roots, int64_t nt)
{
    if (nt < 1) nt = 1;
    orc_forest *f = (orc_forest *)calloc(1, sizeof(orc_forest));
    if (!f) return NULL;
    f->nv = nv; f->nk = nk; f->nt = nt; f->nt_active = nt;
    f->roots = (int64_t *)malloc((size_t)nk * sizeof(int64_t));
    memcpy(f->roots, roots, (size_t)nk * sizeof(int64_t));
    size_t cells = (size_t)nk * (size_t)nv;
    f->level = (int64_t *)malloc(cells * sizeof(int64_t));
    f->sigma = (int64_t *)malloc(cells * sizeof(int64_t));
    f->delta = (double *)malloc(cells * sizeof(double));
    f->bc = (double *)calloc((size_t)nv, sizeof(double));
    f->scr = (orc_scratch *)calloc((size_t)nt, sizeof(orc_scratch));
    if (!f->level || !f->sigma || !f->delta || !f->bc || !f->scr) return NULL;
    for (int64_t t = 0; t < nt; t++) scratch_init(&f->scr[t], nv);
    return f;
}

void orc_forest_free(orc_forest *f)
{
    if (!f) return;
    for (int64_t t = 0; t < f->nt; t++) scratch_free(&f->scr[t]);
    free(f->scr); free(f->roots); free(f->level); free(f->sigma); free(f->delta); free(f->bc);
    free(f);
}

/* Threads used by the following calls (1 .. the count the forest was made
 * with): the reference's NT, which its COARSE loop hands to
 * omp_set_num_threads (src/streamingbc.c:168). */
void orc_set_threads(orc_forest *f, int64_t nt)
{
    f->nt_active = nt < 1 ? 1 : (nt > f->nt ? f->nt : nt);
}

int64_t *orc_forest_level(orc_forest *f) { return f->level; }
int64_t *orc_forest_sigma(orc_forest *f) { return f->sigma; }
double *orc_forest_delta(orc_forest *f) { return f->delta; }
double *orc_forest_bc(orc_forest *f) { return f->bc; }

void orc_forest_counters(const orc_forest *f, int64_t *out4)
{
    out4[0] = f->last_tv; out4[1] = f->last_te; out4[2] = f->last_case1; out4[3] = f->last_case2;
}

/* Fold per-thread BC partials into the forest BC, O(NV*NT) like
 * src/streamingbc.c:211-218 and src/streamingbc_init.c:76-83. */
static void reduce_bc(orc_forest *f)
{
    /* only the active threads' partials can be nonzero: every call clears
     * the partials it folds, so a later call with fewer threads sees zeros */
    int64_t nv = f->nv, nt = f->nt_active;
    #pragma omp parallel for num_threads(nt)
    for (int64_t v = 0; v < nv; v++) {
        for (int64_t t = 0; t < nt; t++) {
            f->bc[v] += f->scr[t].bcpart[v];
            f->scr[t].bcpart[v] = 0.0;
        }
    }
    f->last_tv = f->last_te = f->last_case1 = f->last_case2 = 0;
    for (int64_t t = 0; t < nt; t++) {
        f->last_tv += f->scr[t].tv; f->last_te += f->scr[t].te;
        f->last_case1 += f->scr[t].n1; f->last_case2 += f->scr[t].n2;
        f->scr[t].tv = f->scr[t].te = f->scr[t].n1 = f->scr[t].n2 = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Static Brandes pass for one root (src/streamingbc_init.c:87-183).         */
/* ------------------------------------------------------------------------ */

static void static_root(const orc_graph *g, orc_forest *f, int64_t r, orc_scratch *s)
{
    const int64_t nv = f->nv, root = f->roots[r];
    int64_t *lv = f->level + r * nv;
    int64_t *sg = f->sigma + r * nv;
    double *dl = f->delta + r * nv;

    for (int64_t x = 0; x < nv; x++) { lv[x] = ORC_INF; sg[x] = ORC_INF; dl[x] = 0.0; }
    lv[root] = 0;
    sg[root] = 1;

    /* Forward BFS.  The visit order doubles as the reverse-pass stack. */
    int64_t *order = s->qdown;
    int64_t head = 0, tail = 0;
    order[tail++] = root;
    while (head < tail) {
        int64_t x = order[head++];
        const int64_t *nb = g->nbr[x];
        for (int64_t i = 0; i < g->deg[x]; i++) {
            int64_t k = nb[i];
            if (lv[k] > lv[x]) {                       /* init.c:122 */
                if (lv[k] == ORC_INF) {                /* first discovery, init.c:126-130 */
                    lv[k] = lv[x] + 1;
                    order[tail++] = k;
                }
                if (sg[k] == ORC_INF) sg[k] = sg[x];   /* init.c:132-138 */
                else sg[k] += sg[x];
            }
        }
        s->tv++; s->te += g->deg[x];
    }

    /* Dependency accumulation, deepest first (init.c:155-180). */
    for (int64_t i = tail - 1; i >= 0; i--) {
        int64_t x = order[i];
        const int64_t *nb = g->nbr[x];
        for (int64_t j = 0; j < g->deg[x]; j++) {
            int64_t k = nb[j];
            if (lv[k] == lv[x] - 1)
                dl[k] += ((double)sg[k] / (double)sg[x]) * (dl[x] + 1.0);
        }
        s->tv++; s->te += g->deg[x];
        if (x != root) s->bcpart[x] += dl[x];
    }
}

void orc_static(orc_forest *f, const orc_graph *g)
{
    for (int64_t v = 0; v < f->nv; v++) f->bc[v] = 0.0;
    #pragma omp parallel for schedule(dynamic, 1) num_threads(f->nt_active)
    for (int64_t r = 0; r < f->nk; r++)
        static_root(g, f, r, &f->scr[omp_get_thread_num()]);
    reduce_bc(f);
}

/* ------------------------------------------------------------------------ */
/* |d| == 1: sigma-only descent + dependency ascent                          */
/* (src/streamingbc_internal.c:11-248).  b = deeper endpoint ("start"),      */
/* a = shallower endpoint ("parent"), added = sigma[a].                      */
/* ------------------------------------------------------------------------ */

static void insert_adjacent(const orc_graph *g, orc_forest *f, int64_t r,
                            int64_t b, int64_t a, int64_t added, orc_scratch *s)
{
    const int64_t nv = f->nv, root = f->roots[r];
    int64_t *lv = f->level + r * nv;
    int64_t *sg = f->sigma + r * nv;
    double *dl = f->delta + r * nv;
    int64_t *touched = s->touched, *diff = s->diff, *nsig = s->nsig;
    double *nd = s->ndelta;

    nsig[b] = sg[b] + added;                    /* internal.c:22,28-29 */
    diff[b] = added;
    touched[b] = 1;

    /* Descent: children are neighbours one level deeper (internal.c:53-119). */
    int64_t *qd = s->qdown;
    int64_t head = 0, tail = 0;
    qd[tail++] = b;
    while (head < tail) {
        int64_t x = qd[head++];
        int64_t lx1 = lv[x] + 1;
        int64_t t1 = touched[x] + 1;
        const int64_t *nb = g->nbr[x];
        for (int64_t i = 0; i < g->deg[x]; i++) {
            int64_t k = nb[i];
            if (lv[k] != lx1) continue;
            if (touched[k] == 0) {
                nsig[k] += sg[k];
                qd[tail++] = k;
                touched[k] += t1;
            }
            nsig[k] += diff[x];
            diff[k] += diff[x];
        }
        s->tv++; s->te += g->deg[x];
    }

    /* Ascent: deepest first over Down (reversed) merged with Up (FIFO)
     * (internal.c:138-211). */
    int64_t *qu = s->qup;
    int64_t dn = tail - 1, us = 0, ue = 0;
    while (dn >= 0 || us < ue) {
        int64_t x;
        if (dn < 0) x = qu[us++];
        else if (us < ue && !(lv[qu[us]] < lv[qd[dn]])) x = qu[us++];
        else x = qd[dn--];

        int64_t lm1 = lv[x] - 1;
        const int64_t *nb = g->nbr[x];
        for (int64_t i = 0; i < g->deg[x]; i++) {
            int64_t k = nb[i];
            if (lv[k] != lm1) continue;
            if (touched[k] == 0) {
                nd[k] += dl[k];
                touched[k] = -1;
                qu[ue++] = k;
                nsig[k] += sg[k];
            }
            nd[k] += ((double)nsig[k] / (double)nsig[x]) * (nd[x] + 1.0);
            if (touched[k] < 0 && (k != a || x != b))
                nd[k] -= ((double)sg[k] / (double)sg[x]) * (dl[x] + 1.0);
        }
        s->tv++; s->te += g->deg[x];
        if (x != root) s->bcpart[x] += nd[x] - dl[x];
    }

    /* Commit and reset scratch of touched vertices only (internal.c:213-247). */
    for (int64_t c = 0; c < tail; c++) {
        int64_t k = qd[c];
        dl[k] = nd[k];
        sg[k] = nsig[k];
        diff[k] = 0; touched[k] = 0; nd[k] = 0.0; nsig[k] = 0;
    }
    for (int64_t c = 0; c < ue; c++) {
        int64_t k = qu[c];
        dl[k] = nd[k];
        diff[k] = 0; touched[k] = 0; nd[k] = 0.0; nsig[k] = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* |d| > 1: re-levelling descent + three-queue ascent                       */
/* (src/streamingbc_internal.c:251-603).  b moves up to level[a] + 1.        */
/* ------------------------------------------------------------------------ */

static void bucket_append(orc_scratch *s, int64_t level, int64_t x)
{
    int64_t n = s->bsize++;
    s->bdata[n] = x;
    s->bnext[n] = -1;
    if (s->bback[level] == -1) s->bfront[level] = n;
    else s->bnext[s->bback[level]] = n;
    s->bback[level] = n;
}

static void insert_moving(const orc_graph *g, orc_forest *f, int64_t r,
                          int64_t b, int64_t a, orc_scratch *s)
{
    const int64_t nv = f->nv, root = f->roots[r];
    int64_t *lv = f->level + r * nv;
    int64_t *sg = f->sigma + r * nv;
    double *dl = f->delta + r * nv;
    int64_t *touched = s->touched, *diff = s->diff, *nsig = s->nsig, *nl = s->nlev;
    int64_t *moved = s->moved;
    double *nd = s->ndelta;

    nsig[a] = sg[a];                            /* internal.c:266-283 */
    nsig[b] = sg[a];
    diff[b] = sg[a];
    nl[b] = lv[a] + 1;
    moved[b] = 1;
    touched[b] = 1;

    /* Descent in BFS order of the new tree (internal.c:294-386). */
    int64_t *qd = s->qdown;
    int64_t head = 0, tail = 0;
    qd[tail++] = b;
    while (head < tail) {
        int64_t x = qd[head++];
        int64_t t1 = touched[x] + 1;
        const int64_t *nb = g->nbr[x];
        for (int64_t i = 0; i < g->deg[x]; i++) {
            int64_t k = nb[i];
            if (touched[k] == 0) {
                int64_t c = lv[k] - nl[x] - 1;   /* movement of k via x */
                touched[k] = t1;
                if (c > 0) {
                    nsig[k] = diff[x];
                    diff[k] = diff[x];
                    nl[k] = nl[x] + 1;
                    moved[k] = 1;
                    qd[tail++] = k;
                } else if (c == 0) {
                    nsig[k] = sg[k] + diff[x];
                    diff[k] += diff[x];
                    nl[k] = lv[k];
                    moved[k] = 0;
                    qd[tail++] = k;
                } else {
                    touched[k] = 0;
                }
            } else if (touched[k] == t1) {
                int64_t c = lv[k] - nl[x] - 1;
                if (c >= 0) {
                    nsig[k] += diff[x];
                    diff[k] += diff[x];
                }
            }
        }
        s->tv++; s->te += g->deg[x];
        lv[x] = nl[x];                           /* internal.c:370-371 */
        bucket_append(s, lv[x], x);
    }

    /* Drain the level buckets from the start vertex's level up to NV
     * (internal.c:392-400): O(NV) in the reference, kept here. */
    int64_t nd_cnt = 0;
    for (int64_t lev = lv[b]; lev < nv; lev++) {
        int64_t n = s->bfront[lev];
        while (n != -1) {
            qd[nd_cnt++] = s->bdata[n];
            n = s->bnext[n];
        }
        s->bfront[lev] = -1;
        s->bback[lev] = -1;
    }
    s->bsize = 0;

    /* Three-queue ascent, deepest first; ties go Down, then Up, then Same
     * (internal.c:427-545). */
    int64_t *qu = s->qup, *qs = s->qsame;
    int64_t dn = nd_cnt - 1, us = 0, ue = 0, ss = 0, se = 0;
    for (;;) {
        int64_t dD = dn >= 0 ? lv[qd[dn]] : -1;
        int64_t dU = us < ue ? lv[qu[us]] : -1;
        int64_t dS = ss < se ? lv[qs[ss]] : -1;
        if (dD == -1 && dU == -1 && dS == -1) break;
        int64_t x;
        if (dD >= dS && dD >= dU) x = qd[dn--];
        else if (dU >= dS && dU >= dD) x = qu[us++];
        else x = qs[ss++];

        int64_t lx = lv[x], lm1 = lx - 1;
        const int64_t *nb = g->nbr[x];
        for (int64_t i = 0; i < g->deg[x]; i++) {
            int64_t k = nb[i];
            if (lv[k] == lm1) {
                if (touched[k] == 0) {
                    nd[k] = dl[k];
                    touched[k] = -1;
                    qu[ue++] = k;
                    nsig[k] = sg[k];
                }
                nd[k] += ((double)nsig[k] / (double)nsig[x]) * (nd[x] + 1.0);
                if (touched[k] < 0 && (k != a || x != b))
                    nd[k] -= ((double)sg[k] / (double)sg[x]) * (dl[x] + 1.0);
            } else if (lv[k] == lx && moved[x] == 1 && moved[k] < 0) {
                /* k kept its level and lost x as a child (internal.c:509-533) */
                if (touched[k] == 0) {
                    nd[k] = dl[k];
                    touched[k] = -2;
                    qs[se++] = k;
                    nsig[k] = sg[k];
                }
                nd[k] -= ((double)sg[k] / (double)sg[x]) * (dl[x] + 1.0);
            }
        }
        s->tv++; s->te += g->deg[x];
        if (x != root) s->bcpart[x] += nd[x] - dl[x];
    }

    /* Commit and reset (internal.c:547-602). */
    for (int64_t c = 0; c < nd_cnt; c++) {
        int64_t k = qd[c];
        dl[k] = nd[k];
        sg[k] = nsig[k];
        diff[k] = 0; touched[k] = 0; nd[k] = 0.0; nl[k] = 0; moved[k] = -1; nsig[k] = 0;
    }
    for (int64_t c = 0; c < se; c++) {
        int64_t k = qs[c];
        dl[k] = nd[k];
        diff[k] = 0; touched[k] = 0; nd[k] = 0.0; moved[k] = -1; nsig[k] = 0;
    }
    for (int64_t c = 0; c < ue; c++) {
        int64_t k = qu[c];
        dl[k] = nd[k];
        diff[k] = 0; touched[k] = 0; nd[k] = 0.0; moved[k] = -1; nsig[k] = 0;
    }
}

/* ------------------------------------------------------------------------ */
/* Dispatcher (src/streamingbc.c:88-226, COARSE branch at :168-208).         */
/* The caller inserts (u,v) and (v,u) into the graph first.                  */
/* ------------------------------------------------------------------------ */

static void insert_root(const orc_graph *g, orc_forest *f, int64_t r,
                        int64_t u, int64_t v, orc_scratch *s)
{
    const int64_t nv = f->nv;
    const int64_t *lv = f->level + r * nv;
    const int64_t *sg = f->sigma + r * nv;
    int64_t lu = lv[u], lvv = lv[v];
    if (lu == lvv) return;                      /* same level or both unreachable */
    /* b = deeper endpoint; an unreachable endpoint counts as deepest */
    int64_t b = lu > lvv ? u : v;
    int64_t a = lu > lvv ? v : u;
    int64_t gap = lv[b] - lv[a];                /* no overflow: lv[a] >= 0 */
    if (gap == 1) {
        insert_adjacent(g, f, r, b, a, sg[a], s);
        s->n1++;
    } else {
        insert_moving(g, f, r, b, a, s);
        s->n2++;
    }
}

void orc_insert(orc_forest *f, const orc_graph *g, int64_t u, int64_t v)
{
    #pragma omp parallel for schedule(dynamic, 1) num_threads(f->nt_active)
    for (int64_t r = 0; r < f->nk; r++)
        insert_root(g, f, r, u, v, &f->scr[omp_get_thread_num()]);
    reduce_bc(f);
}

/* orc_insert with its two phases timed (wall seconds): the per-root updates
 * (scale with the number of roots) and the per-thread BC reduce (O(NV*NT),
 * independent of the number of roots). */
void orc_insert_timed(orc_forest *f, const orc_graph *g, int64_t u, int64_t v, double *t_roots, double *t_reduce)
{
    double t0 = omp_get_wtime();
    #pragma omp parallel for schedule(dynamic, 1) num_threads(f->nt_active)
    for (int64_t r = 0; r < f->nk; r++)
        insert_root(g, f, r, u, v, &f->scr[omp_get_thread_num()]);
    double t1 = omp_get_wtime();
    reduce_bc(f);
    double t2 = omp_get_wtime();
    *t_roots = t1 - t0;
    *t_reduce = t2 - t1;
}

/* Static init timed (wall seconds). */
double orc_static_timed(orc_forest *f, const orc_graph *g)
{
    double t0 = omp_get_wtime();
    for (int64_t x = 0; x < f->nv; x++) f->bc[x] = 0.0;
    #pragma omp parallel for schedule(dynamic, 1) num_threads(f->nt_active)
    for (int64_t r = 0; r < f->nk; r++)
        static_root(g, f, r, &f->scr[omp_get_thread_num()]);
    reduce_bc(f);
    return omp_get_wtime() - t0;
}

/* Per-insertion classification of every root at the current state:
 * out[r] = 0 (same level / both unreachable), 1 (|d| == 1), 2 (|d| > 1). */
void orc_classify(const orc_forest *f, int64_t u, int64_t v, int8_t *out)
{
    const int64_t nv = f->nv;
    for (int64_t r = 0; r < f->nk; r++) {
        int64_t lu = f->level[r * nv + u], lvv = f->level[r * nv + v];
        if (lu == lvv) out[r] = 0;
        else {
            int64_t hi = lu > lvv ? lu : lvv, lo = lu > lvv ? lvv : lu;
            out[r] = (hi - lo == 1) ? 1 : 2;
        }
    }
}
