/*
 * streamingbc.h -- drop-in for the reference's public BC API
 * (src/streamingbc.h:38-64 of ogreen/StreamingBC), implemented by
 * libsbc_gb300.so over GB300 kernels.
 *
 * Same names, argument meaning and call order as the reference:
 *   forest = streamingBCCreateForestApproximate(NV, NK, roots);
 *   aux    = streamingBCCreateAuxilary(NT, NV);
 *   streamingBCInitStaticApproximate(forest, G, NT, aux, NK, roots);
 *   stinger_insert_edge(G, 0, u, v, 0, 0); stinger_insert_edge(G, 0, v, u, 0, 0);
 *   insertEdgeStreamingBC(forest, G, u, v, roots, NK, NV, NT, aux, BALANCE, COARSE);
 *
 * Documented differences:
 *   - Per-root state lives in GPU memory.  forest->totalBC is a host mirror,
 *     refreshed after every static init and insertion call.  The per-tree host
 *     records forest->forest[root]->vArr[v] are only filled by the added call
 *     streamingBCSyncForest(forest); their edgesAbove/edgesBelow are 0 (those
 *     fields only drive the BALANCE ordering, src/streamingbc.c:104-122).
 *   - NT, loadBalancing and granularity are accepted and ignored: results never
 *     depend on them, and FINE (src/streamingbc_internal_fine.c) is not a
 *     separate code path.
 *   - insertEdgeStreamingBC returns real per-call counts in StreamingExtraInfo
 *     (movement = roots with |d| > 1, adjacent = roots with |d| == 1,
 *     sameLevel = roots left unchanged); the reference returns zeros.  The
 *     counters of aux[0] receive the reference's traversal counters.
 *   - deleteEdgeStreamingBC (after the caller's stinger_remove_edge x2, as in
 *     the reference) ends in the state of the modified graph -- the same as a
 *     static recompute -- which the reference's own deletion does not; its
 *     counts are adjacent = roots updated incrementally, movement = roots
 *     recomputed.  deleteVertexStreamingBC deletes the vertex's edges one at
 *     a time the same way and reports the former neighbours in
 *     adjacencyArray / *adjacencySize (the reference leaves the size at 0).
 *   - Failures do not abort: functions keep their reference signatures and
 *     report through sbc_last_error() (NULL / zero results on failure).
 */
#ifndef SBC_STREAMINGBC_H_
#define SBC_STREAMINGBC_H_

#include <stdint.h>
#include "stinger.h"
#include "sbc_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef double bc_t;

/* src/streamingbc_aux.h:21-27 */
typedef struct {
    int64_t level;
    int64_t sigma;
    int64_t edgesBelow;
    int64_t edgesAbove;
    bc_t delta;
} bcV;

/* src/streamingbc_aux.h:29-33 */
typedef struct {
    int64_t NV;
    bcV *vArr;
} bcTree;
typedef bcTree *bcTreePtr;

/* src/streamingbc_aux.h:35-40; the first three fields keep the reference
 * layout, the rest belong to this implementation. */
typedef struct {
    bcTreePtr *forest; /* indexed by root vertex id; filled by streamingBCSyncForest */
    bc_t *totalBC;     /* host mirror of BC */
    int64_t NV;
    sbc_forest *sbc;   /* device forest (created at the first static init) */
    int64_t sbc_nk;
    int64_t *sbc_roots;
} bcForest;
typedef bcForest *bcForestPtr;

/* src/streamingbc_aux.h:42-48 */
typedef struct {
    int64_t movement;
    int64_t adjacent;
    int64_t sameLevel;
    int64_t connectedComponents;
} StreamingExtraInfo;

/* Counter part of src/streamingbc_aux.h:147-188.  The scratch arrays of the
 * reference live on the GPU (per persistent worker), not here. */
typedef struct {
    int64_t samelevelCounter;
    int64_t compConnCounter;
    int64_t adjacentCounter;
    int64_t movementCounter;
    int64_t staticTraverseVerticeCounter;
    int64_t staticTraverseEdgeCounter;
    int64_t dynamicTraverseVerticeCounter;
    int64_t dynamicTraverseEdgeCounter;
} extraArraysPerThread;

/* src/streamingbc.h:9-27 */
typedef enum { COARSE, FINE } granularity_t;
typedef enum { DELETE, INSERT } operation_t;
typedef enum { NO_BALANCE, BALANCE } lbalance_t;
typedef enum { UP_INSERT = 0, UP_DELETE } updateType;

/* src/streamingbc.h:30-35 */
typedef struct {
    int64_t NV;
    int64_t NE;
    int64_t *edgeArray;
    int64_t *vertexPointerArray;
} csrGraph;

/* ---- src/streamingbc.h:40-44: forest creation and destruction ---- */
bcForest *streamingBCCreateForestExact(int64_t NV);
bcForest *streamingBCCreateForestApproximate(int64_t NV, int64_t NK, int64_t *rootArrayForApproximation);
void streamingBCDeleteForestExact(bcForestPtr *deadForest);
void streamingBCDeleteForestApproximate(bcForestPtr *deadForest, int64_t rootArraySize, int64_t *rootArray);

/* ---- src/streamingbc.h:47-48: auxiliary data ---- */
extraArraysPerThread **streamingBCCreateAuxilary(int64_t threadCount, int64_t NV);
void streamingBCDeleteAuxilary(extraArraysPerThread **parallelExtra, int64_t threadCount, int64_t NV);

/* ---- src/streamingbc.h:51-52: static computation ---- */
void streamingBCInitStaticExact(bcForest *forest, struct stinger *stingerGraph, int64_t NT,
                                extraArraysPerThread **auxilary);
void streamingBCInitStaticApproximate(bcForest *forest, struct stinger *stingerGraph, int64_t NT,
                                      extraArraysPerThread **auxilary, int64_t NK,
                                      int64_t *rootArrayForApproximation);

/* ---- src/streamingbc.h:55-58: edge updates ---- */
StreamingExtraInfo insertEdgeStreamingBC(bcForest *forest, struct stinger *sStinger, int64_t newU, int64_t newV,
                                         int64_t *rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                         extraArraysPerThread **eAPT, uint32_t loadBalancing,
                                         uint32_t granularity);
StreamingExtraInfo deleteEdgeStreamingBC(bcForest *forest, struct stinger *sStinger, int64_t oldU, int64_t oldV,
                                         int64_t *rootArrayForApproximation, int64_t NK, int64_t Nv, int64_t NT,
                                         extraArraysPerThread **eAPT, uint32_t loadBalancing,
                                         uint32_t granularity);

/* ---- src/streamingbc.h:61-64: vertex updates ---- */
StreamingExtraInfo insertVertexStreamingBC(bcForest *forest, struct stinger *sStinger, int64_t src,
                                           int64_t *adjacencyArray, int64_t adjacencySize,
                                           int64_t *rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                           extraArraysPerThread **eAPT);
StreamingExtraInfo deleteVertexStreamingBC(bcForest *forest, struct stinger *sStinger, int64_t src,
                                           int64_t *adjacencyArray, int64_t *adjacencySize,
                                           int64_t *rootArrayForApproximation, int64_t NK, int64_t NV, int64_t NT,
                                           extraArraysPerThread **eAPT);

/* ---- src/streamingbc.h:67-73: CSR helpers of the reference driver ---- */
void CreateStingerFromCSR(csrGraph *csr, struct stinger **stingerGraph);
csrGraph *CreateEmptyUndirectedCSR(int64_t NV, int64_t NE);
csrGraph *CreateEmptyDirectedCSR(int64_t NV, int64_t NE);
void FreeCSR(csrGraph *graph);
/* src/streamingbc.h:84 (src/sbcMain_utils.c:382-422): a DIMACS .graph file
 * into a new device graph; *NV counts the unused vertex 0 (header NV + 1) and
 * *NE is the header's NE doubled, as in the reference.  The file is parsed by
 * all host threads and the adjacency built on the device; on failure
 * *stingerGraph is NULL and sbc_last_error() says why (the reference would
 * crash). */
void ParseDimacsGraph(char initial_graph_name[1024], struct stinger **stingerGraph, int64_t *NV, int64_t *NE);
/* src/sbcMain_utils.c:425-456: identity when NK == NV, else NK distinct
 * vertices drawn with rand() (seed with srand). */
void PickRoots(int64_t *rootArrayForApproximation, int64_t NK, int64_t NV);
/* src/streamingbc_aux.c:305-317 */
void ClearCounters(extraArraysPerThread *eapt);

/* ---- added: fill forest->forest[root]->vArr from the device state ---- */
int streamingBCSyncForest(bcForest *forest);

#ifdef __cplusplus
}
#endif

#endif /* SBC_STREAMINGBC_H_ */
