/*
 * The reference driver's own flow (src/sbcMain.c:63-101) through the drop-in
 * headers: ParseDimacsGraph -> srand + PickRoots -> forest + auxiliary arrays
 * -> static init, then insertions the way updateEdgeNEW applies them
 * (src/sbcMain_utils.c:556-574: stinger_insert_edge x2, insertEdgeStreamingBC).
 * Compiled with plain gcc; nothing in it knows about CUDA.
 *
 * usage: dimacs_driver <graph.graph> <NK> <insertions> <output>
 *   insertions: text "NI", then NI pairs "u v" (file ids, 1-based)
 *   output: "nv <NV> ne <NE>", then after static init and after each insertion
 *           one line "bc <i> <NV doubles>"
 */
#include <stdio.h>
#include <stdlib.h>
#include "streamingbc.h"
#include "stinger.h"

static void dump(FILE *out, long long i, const bcForest *forest, int64_t NV)
{
    fprintf(out, "bc %lld", i);
    for (int64_t v = 0; v < NV; v++) fprintf(out, " %.17g", forest->totalBC[v]);
    fprintf(out, "\n");
}

int main(int argc, char **argv)
{
    if (argc != 5) return 2;
    char name[1024];
    snprintf(name, sizeof name, "%s", argv[1]);
    const long long NK_arg = atoll(argv[2]);
    FILE *ins = fopen(argv[3], "r");
    FILE *out = fopen(argv[4], "w");
    if (!ins || !out) return 2;

    struct stinger *G = NULL;
    int64_t NV = 0, NE = 0;
    ParseDimacsGraph(name, &G, &NV, &NE);
    if (!G) {
        fprintf(stderr, "parse: %s\n", sbc_last_error());
        return 3;
    }
    const int64_t NK = NK_arg > 0 && NK_arg < NV ? NK_arg : NV;
    srand(1);
    int64_t *roots = (int64_t *)malloc(sizeof(int64_t) * (size_t)NK);
    PickRoots(roots, NK, NV);
    fprintf(out, "nv %lld ne %lld\n", (long long)NV, (long long)NE);

    const int64_t NT = 4;
    bcForest *forest = streamingBCCreateForestApproximate(NV, NK, roots);
    extraArraysPerThread **aux = streamingBCCreateAuxilary(NT, NV);
    streamingBCInitStaticApproximate(forest, G, NT, aux, NK, roots);
    if (sbc_last_error()[0]) {
        fprintf(stderr, "static: %s\n", sbc_last_error());
        return 4;
    }
    dump(out, -1, forest, NV);

    long long NI = 0;
    if (fscanf(ins, "%lld", &NI) != 1) return 5;
    for (long long i = 0; i < NI; i++) {
        long long u, v;
        if (fscanf(ins, "%lld %lld", &u, &v) != 2) return 5;
        stinger_insert_edge(G, 0, u, v, 0, 0);
        stinger_insert_edge(G, 0, v, u, 0, 0);
        insertEdgeStreamingBC(forest, G, u, v, roots, NK, NV, NT, aux, BALANCE, COARSE);
        if (sbc_last_error()[0]) {
            fprintf(stderr, "insert %lld: %s\n", i, sbc_last_error());
            return 6;
        }
        dump(out, i, forest, NV);
    }
    streamingBCDeleteAuxilary(aux, NT, NV);
    streamingBCDeleteForestApproximate(&forest, NK, roots);
    stinger_free(G);
    free(roots);
    fclose(out);
    fclose(ins);
    return 0;
}
