/*
 * A reference-style caller of the streamingbc.h API, written exactly as the
 * reference's own driver uses it (src/sbcMain.c, src/sbcMain_utils.c:306-338,
 * :458-471): CSR -> CreateStingerFromCSR -> forest + auxiliary arrays -> static
 * init -> for each insertion: stinger_insert_edge x2, insertEdgeStreamingBC;
 * then for each deletion: stinger_remove_edge x2, deleteEdgeStreamingBC;
 * then optionally deleteVertexStreamingBC of one vertex, then optionally
 * insertVertexStreamingBC of one vertex with a list of neighbours.
 * Compiled with plain gcc against include/streamingbc.h and linked to
 * libsbc_gb300.so; nothing in it knows about CUDA.
 *
 * usage: drop_in_driver <input> <output>
 *   input : text "NV NE NK NI", then NV+1 offsets, NE neighbour ids,
 *           NK roots, NI pairs "u v"
 *   output: text, after static init and after each insertion one line
 *           "bc <i> <NV doubles>", then the final levels and sigmas of every
 *           root ("lv <r> ...", "sg <r> ...") read through forest->forest[root].
 */
#include <stdio.h>
#include <stdlib.h>
#include "streamingbc.h"

int main(int argc, char **argv)
{
    if (argc != 3) return 2;
    FILE *in = fopen(argv[1], "r");
    FILE *out = fopen(argv[2], "w");
    if (!in || !out) return 2;
    long long NV, NE, NK, NI;
    if (fscanf(in, "%lld %lld %lld %lld", &NV, &NE, &NK, &NI) != 4) return 3;
    csrGraph *csr = CreateEmptyDirectedCSR(NV, NE);
    for (long long v = 0; v <= NV; v++) {
        long long x;
        if (fscanf(in, "%lld", &x) != 1) return 3;
        csr->vertexPointerArray[v] = x;
    }
    for (long long e = 0; e < NE; e++) {
        long long x;
        if (fscanf(in, "%lld", &x) != 1) return 3;
        csr->edgeArray[e] = x;
    }
    int64_t *roots = (int64_t *)malloc(sizeof(int64_t) * (size_t)NK);
    for (long long r = 0; r < NK; r++) {
        long long x;
        if (fscanf(in, "%lld", &x) != 1) return 3;
        roots[r] = x;
    }
    struct stinger *G;
    CreateStingerFromCSR(csr, &G);
    FreeCSR(csr);

    const int64_t NT = 4;
    bcForest *forest = streamingBCCreateForestApproximate(NV, NK, roots);
    extraArraysPerThread **aux = streamingBCCreateAuxilary(NT, NV);
    streamingBCInitStaticApproximate(forest, G, NT, aux, NK, roots);
    if (sbc_last_error()[0]) {
        fprintf(stderr, "static: %s\n", sbc_last_error());
        return 4;
    }
    fprintf(out, "bc -1");
    for (long long v = 0; v < NV; v++) fprintf(out, " %.17g", forest->totalBC[v]);
    fprintf(out, "\n");

    for (long long i = 0; i < NI; i++) {
        long long u, v;
        if (fscanf(in, "%lld %lld", &u, &v) != 2) return 3;
        stinger_insert_edge(G, 0, u, v, 0, 0);
        stinger_insert_edge(G, 0, v, u, 0, 0);
        insertEdgeStreamingBC(forest, G, u, v, roots, NK, NV, NT, aux, BALANCE, COARSE);
        fprintf(out, "bc %lld", i);
        for (long long x = 0; x < NV; x++) fprintf(out, " %.17g", forest->totalBC[x]);
        fprintf(out, "\n");
    }
    if (streamingBCSyncForest(forest) != 0) {
        fprintf(stderr, "sync: %s\n", sbc_last_error());
        return 5;
    }
    for (long long r = 0; r < NK; r++) {
        bcTree *t = forest->forest[roots[r]];
        fprintf(out, "lv %lld", r);
        for (long long x = 0; x < NV; x++) fprintf(out, " %lld", (long long)t->vArr[x].level);
        fprintf(out, "\nsg %lld", r);
        for (long long x = 0; x < NV; x++) fprintf(out, " %lld", (long long)t->vArr[x].sigma);
        fprintf(out, "\n");
    }
    fprintf(out, "degree0 %lld\n", (long long)stinger_outdegree(G, 0));

    /* optional tail: deletions, as the reference's callers make them
     * (stinger_remove_edge x2, then deleteEdgeStreamingBC) */
    long long ND = 0;
    if (fscanf(in, "%lld", &ND) != 1) ND = 0;
    for (long long i = 0; i < ND; i++) {
        long long u, v;
        if (fscanf(in, "%lld %lld", &u, &v) != 2) return 3;
        if (stinger_remove_edge(G, 0, u, v) != 1 || stinger_remove_edge(G, 0, v, u) != 1) return 6;
        deleteEdgeStreamingBC(forest, G, u, v, roots, NK, NV, NT, aux, BALANCE, COARSE);
        if (sbc_last_error()[0]) {
            fprintf(stderr, "delete: %s\n", sbc_last_error());
            return 7;
        }
        fprintf(out, "dbc %lld", i);
        for (long long x = 0; x < NV; x++) fprintf(out, " %.17g", forest->totalBC[x]);
        fprintf(out, "\n");
    }

    /* optional: delete a whole vertex (deleteVertexStreamingBC) */
    long long VD = -1;
    if (fscanf(in, "%lld", &VD) != 1) VD = -1;
    if (VD >= 0) {
        int64_t *adj = (int64_t *)malloc(sizeof(int64_t) * (size_t)NV);
        int64_t size = -1;
        deleteVertexStreamingBC(forest, G, VD, adj, &size, roots, NK, NV, NT, aux);
        if (sbc_last_error()[0]) {
            fprintf(stderr, "delete vertex: %s\n", sbc_last_error());
            return 8;
        }
        fprintf(out, "vdeg %lld %lld\n", (long long)size, (long long)stinger_outdegree(G, VD));
        fprintf(out, "vbc 0");
        for (long long x = 0; x < NV; x++) fprintf(out, " %.17g", forest->totalBC[x]);
        fprintf(out, "\n");
        free(adj);
    }

    /* optional: insert a vertex's edges (insertVertexStreamingBC inserts them
     * into the graph itself, src/streamingbc.c:56-77) */
    long long VI = -1, NVI = 0;
    if (fscanf(in, "%lld %lld", &VI, &NVI) != 2) VI = -1;
    if (VI >= 0) {
        int64_t *adj = (int64_t *)malloc(sizeof(int64_t) * (size_t)(NVI > 0 ? NVI : 1));
        for (long long i = 0; i < NVI; i++) {
            long long x;
            if (fscanf(in, "%lld", &x) != 1) return 3;
            adj[i] = x;
        }
        StreamingExtraInfo sei = insertVertexStreamingBC(forest, G, VI, adj, NVI, roots, NK, NV, NT, aux);
        if (sbc_last_error()[0]) {
            fprintf(stderr, "insert vertex: %s\n", sbc_last_error());
            return 9;
        }
        fprintf(out, "ivdeg %lld %lld %lld\n", (long long)stinger_outdegree(G, VI), (long long)sei.adjacent,
                (long long)sei.movement);
        fprintf(out, "ivbc 0");
        for (long long x = 0; x < NV; x++) fprintf(out, " %.17g", forest->totalBC[x]);
        fprintf(out, "\n");
        if (streamingBCSyncForest(forest) != 0) {
            fprintf(stderr, "sync: %s\n", sbc_last_error());
            return 5;
        }
        for (long long r = 0; r < NK; r++) {
            bcTree *t = forest->forest[roots[r]];
            fprintf(out, "ivlv %lld", r);
            for (long long x = 0; x < NV; x++) fprintf(out, " %lld", (long long)t->vArr[x].level);
            fprintf(out, "\nivsg %lld", r);
            for (long long x = 0; x < NV; x++) fprintf(out, " %lld", (long long)t->vArr[x].sigma);
            fprintf(out, "\n");
        }
        free(adj);
    }
    streamingBCDeleteAuxilary(aux, NT, NV);
    streamingBCDeleteForestApproximate(&forest, NK, roots);
    stinger_free(G);
    free(roots);
    fclose(out);
    fclose(in);
    return 0;
}
