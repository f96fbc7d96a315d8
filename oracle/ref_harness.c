/*
 * Harness around the UNMODIFIED reference sources -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiled together with the reference's own C files, read in place from the
 * reference tree, into oracle/_ref/libsbcref.so (see oracle/Makefile).  It
 * drives the reference exactly like its driver does:
 *   graph      CreateEmptyDirectedCSR + CreateStingerFromCSR  (src/sbcMain_utils.c:306-338)
 *   forest     CreateForestApproximate + createExtraArraysForThreads
 *   static     BrandesApproxCaseParallel                    (src/streamingbc_init.c:60-84)
 *   insertion  stinger_insert_edge x2, then insertEdgeStreamingBC(..., BALANCE, COARSE)
 *              (src/sbcMain_utils.c:458-471), counters cleared after each call.
 * It exists to pin the C restatement in sbc_oracle.c and to produce golden
 * vectors; it is never part of the product.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#include "streamingbc.h"
#include "timer.h"

static struct stinger *g_S;
static bcForest *g_F;
static extraArraysPerThread **g_A;
static int64_t g_nv, g_nk, g_nt;
static int64_t *g_roots;
static int64_t g_cnt[4];

int ref_init(int64_t nv, const int64_t *off, const int64_t *adj, int64_t nk, const int64_t *roots, int64_t nt)
{
    csrGraph *c = CreateEmptyDirectedCSR(nv, off[nv]);
    for (int64_t v = 0; v <= nv; v++) c->vertexPointerArray[v] = off[v];
    for (int64_t e = 0; e < off[nv]; e++) c->edgeArray[e] = adj[e];
    CreateStingerFromCSR(c, &g_S);
    FreeCSR(c);
    g_nv = nv; g_nk = nk; g_nt = nt;
    g_roots = (int64_t *)malloc(sizeof(int64_t) * nk);
    memcpy(g_roots, roots, sizeof(int64_t) * nk);
    g_F = CreateForestApproximate(nv, g_roots, nk);
    g_A = createExtraArraysForThreads(nt, nv);
    return 0;
}

double ref_static(void)
{
    tic();
    BrandesApproxCaseParallel(g_F, g_S, g_roots, g_nk, g_A, g_nt);
    double t = toc();
    g_cnt[0] = g_cnt[1] = 0;
    for (int64_t t2 = 0; t2 < g_nt; t2++) {
        g_cnt[0] += g_A[t2]->staticTraverseVerticeCounter;
        g_cnt[1] += g_A[t2]->staticTraverseEdgeCounter;
        ClearCounters(g_A[t2]);
    }
    return t;
}

/* Returns the seconds spent inside insertEdgeStreamingBC, timed like
 * updateEdgeNEW (src/sbcMain_utils.c:568-571). */
double ref_insert(int64_t u, int64_t v)
{
    stinger_insert_edge(g_S, 0, u, v, 0, 0);
    stinger_insert_edge(g_S, 0, v, u, 0, 0);
    tic();
    insertEdgeStreamingBC(g_F, g_S, u, v, g_roots, g_nk, g_nv, g_nt, g_A, BALANCE, COARSE);
    double t = toc();
    g_cnt[0] = g_cnt[1] = g_cnt[2] = g_cnt[3] = 0;
    for (int64_t t2 = 0; t2 < g_nt; t2++) {
        g_cnt[0] += g_A[t2]->dynamicTraverseVerticeCounter;
        g_cnt[1] += g_A[t2]->dynamicTraverseEdgeCounter;
        g_cnt[2] += g_A[t2]->adjacentCounter;
        g_cnt[3] += g_A[t2]->movementCounter;
        ClearCounters(g_A[t2]);
    }
    return t;
}

/* Deletion as the reference's callers do it (src/sbcMain_utils.c:477-484,
 * :586-591): stinger_remove_edge x2, then deleteEdgeStreamingBC(..., BALANCE,
 * COARSE) (src/streamingbc.c:258-416).  Counters as for ref_insert (case1 =
 * adjacent-level deletions, case2 = deletions that move vertices down). */
double ref_delete(int64_t u, int64_t v)
{
    stinger_remove_edge(g_S, 0, u, v);
    stinger_remove_edge(g_S, 0, v, u);
    tic();
    deleteEdgeStreamingBC(g_F, g_S, u, v, g_roots, g_nk, g_nv, g_nt, g_A, BALANCE, COARSE);
    double t = toc();
    g_cnt[0] = g_cnt[1] = g_cnt[2] = g_cnt[3] = 0;
    for (int64_t t2 = 0; t2 < g_nt; t2++) {
        g_cnt[0] += g_A[t2]->dynamicTraverseVerticeCounter;
        g_cnt[1] += g_A[t2]->dynamicTraverseEdgeCounter;
        g_cnt[2] += g_A[t2]->adjacentCounter;
        g_cnt[3] += g_A[t2]->movementCounter;
        ClearCounters(g_A[t2]);
    }
    return t;
}

void ref_counters(int64_t *out4) { memcpy(out4, g_cnt, sizeof(g_cnt)); }

void ref_dump(int64_t *level, int64_t *sigma, double *delta, double *bc)
{
    for (int64_t r = 0; r < g_nk; r++) {
        bcTree *t = g_F->forest[g_roots[r]];
        for (int64_t x = 0; x < g_nv; x++) {
            level[r * g_nv + x] = t->vArr[x].level;
            sigma[r * g_nv + x] = t->vArr[x].sigma;
            delta[r * g_nv + x] = t->vArr[x].delta;
        }
    }
    memcpy(bc, g_F->totalBC, sizeof(double) * g_nv);
}

void ref_free(void)
{
    if (g_A) destroyExtraArraysForThreads(g_A, g_nt, g_nv);
    if (g_F) DestroyForestApproximate(&g_F, g_roots, g_nk);
    if (g_S) stinger_free(g_S);
    free(g_roots);
    g_A = NULL; g_F = NULL; g_S = NULL; g_roots = NULL;
}
